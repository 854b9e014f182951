// Many independent dense SPD systems of uneven sizes, solved by plain FP32 CG in one persistent launch.
//
// Each system follows the reference's run_batched_cg exactly as a separate
// cola.linalg.solve(PSD(Dense(A_s)), b_s, CG(tol, max_iters)) call would (cg.py:94-154):
//   b <- b/|b|, r0 = b, p0 = r0, gamma0 = <r0, r0>, tol_eff = tol*|r0| + tol,
//   steps while |r| > tol_eff and k < max_iters, alpha/beta zeroed once |r| < 1e-40,
//   solution scaled back by |b|.
// Systems converge independently (per-system masks); the rows of the still-active systems are
// re-partitioned over all warps at every phase, so warps stay busy as small systems finish: the
// matvec's rows in chunks of about equal cost (n_s per row) claimed from a counter, the vector
// phases' rows split evenly.
//
// Layout: A_s row-major at vals + a_off[s]; vectors of system s at v_off[s] in concatenated buffers.
// The search direction p of system s is kept in four copies, copy h shifted right by h elements
// (copy h holds p[i] at index i + h, each copy 16-byte aligned).  A row whose first element sits h
// floats past a 16-byte boundary is read as aligned 128-bit quads from its first boundary on, and
// copy h then lines the matching p quads up on 16-byte boundaries as well, so the matvec issues only
// 128-bit loads whatever n_s and the offsets are (the up to 3 + 3 elements before the first and
// after the last whole quad are scalar).  The shifted copies cost 3 extra n_s-float writes a step
// against the n_s^2 floats of A the step reads.
#include <algorithm>
#include <string>

#include "common.cuh"

namespace colagb {

constexpr int kDBThreads = 256;
constexpr int kDBMaxSystems = 1024;
constexpr long long kDBChunk = 16384;  // matvec work claimed at a time: ~64 KB of A

struct DenseBatchArgs {
  int S;
  const int32_t* sizes;
  const int64_t* a_off;
  const int64_t* v_off;
  const float* vals;
  const float* B;
  float* X;
  float *r, *p4, *ap;  // p4: the four shifted copies of p, system s at copy_base(s)
  double* acc;  // [3][S]: <p, Ap>, |r|^2, |b|^2
  unsigned long long* claim;  // the matvec's chunk counter (zero at every phase start)
  int* out_iters;
  int* out_status;
  double tol;
  int max_iters;
  GridBarrier gb;
};

struct DState {
  unsigned char* base;
  int S;
  __device__ __forceinline__ double* f64(int k) const { return reinterpret_cast<double*>(base) + (size_t)k * S; }
  __device__ __forceinline__ float* f32(int k) const { return reinterpret_cast<float*>(base + (size_t)2 * 8 * S) + (size_t)k * S; }
  __device__ __forceinline__ int* i32(int k) const {
    return reinterpret_cast<int*>(base + (size_t)2 * 8 * S) + (size_t)(6 + k) * S;
  }
  __device__ __forceinline__ long long* prefix() const {  // S + 1 cost prefix sums of the active list
    return reinterpret_cast<long long*>(base + (size_t)2 * 8 * S + (size_t)(6 + 4) * 4 * S + 16);
  }
  __device__ __forceinline__ long long* pbase() const { return prefix() + S + 1; }  // S offsets into p4
  __device__ __forceinline__ double& gamma(int s) const { return f64(0)[s]; }
  __device__ __forceinline__ double& mult(int s) const { return f64(1)[s]; }
  __device__ __forceinline__ float& alpha(int s) const { return f32(0)[s]; }
  __device__ __forceinline__ float& beta(int s) const { return f32(1)[s]; }
  __device__ __forceinline__ float& rn(int s) const { return f32(2)[s]; }
  __device__ __forceinline__ float& tol_eff(int s) const { return f32(3)[s]; }
  __device__ __forceinline__ float& conv(int s) const { return f32(4)[s]; }
  __device__ __forceinline__ int& it(int s) const { return i32(0)[s]; }
  __device__ __forceinline__ int& active(int s) const { return i32(1)[s]; }
  __device__ __forceinline__ int* act() const { return i32(2); }
};

static size_t dense_batch_smem(int S) {
  return (size_t)2 * 8 * S + (size_t)10 * 4 * S + 16 + (size_t)8 * (S + 1) + (size_t)8 * S + 64;
}

// Length of one shifted copy of an n-vector: room for index n - 1 + 3, rounded to whole quads.
__host__ __device__ __forceinline__ int64_t pcopy_len(int64_t n) { return ((n + 3) & ~int64_t(3)) + 4; }

// Write element i of p (value v) into all four shifted copies.
__device__ __forceinline__ void put_p(float* P0, int64_t cs, int i, float v) {
  P0[i] = v;
  P0[cs + i + 1] = v;
  P0[2 * cs + i + 2] = v;
  P0[3 * cs + i + 3] = v;
}

__device__ __forceinline__ float4 ld_a4(const float* q) {  // read-only A: no L1 allocation
  float4 v;
  asm("ld.global.nc.L1::no_allocate.v4.f32 {%0, %1, %2, %3}, [%4];"
      : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
      : "l"(q));
  return v;
}

__device__ __forceinline__ float dot4(float4 a, float4 b, float s) {
  s = fmaf(a.x, b.x, s);
  s = fmaf(a.y, b.y, s);
  s = fmaf(a.z, b.z, s);
  return fmaf(a.w, b.w, s);
}

// <A row, p> over one warp; the result is in every lane.  Ar: the row (ns floats); P0: copy 0 of p,
// cs: the copy length.  Each lane keeps eight independent 128-bit loads of A in flight (4 KB per
// warp, four 256-thread blocks per SM): the matvec streams HBM and is bound by how many bytes are in
// flight, not by instructions (four quads per lane and 3 blocks reached 0.46 of the copy bandwidth,
// four quads and 4 blocks 0.64, eight quads and 4 blocks 0.78; an L2 prefetch ahead of the loads
// lowered each).
__device__ __forceinline__ float row_dot(const float* __restrict__ Ar, const float* P0, int64_t cs, int ns,
                                         int lane) {
  const int h = (int)((reinterpret_cast<uintptr_t>(Ar) >> 2) & 3);  // floats past the last 16-byte boundary
  int j0 = (4 - h) & 3;                                              // first element of the first whole quad
  if (j0 > ns) j0 = ns;
  const int nq = (ns - j0) >> 2;
  const int jt = j0 + 4 * nq;
  const float* Aq = Ar + j0;              // 16-byte aligned
  const float* Pq = P0 + h * cs + j0 + h;  // copy h: p[j] at index j + h; j0 + h is 0 or 4
  float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;
  int q = lane;
  for (; q + 224 < nq; q += 256) {
    const float4 a0 = ld_a4(Aq + 4 * q), a1 = ld_a4(Aq + 4 * (q + 32));
    const float4 a2 = ld_a4(Aq + 4 * (q + 64)), a3 = ld_a4(Aq + 4 * (q + 96));
    const float4 a4 = ld_a4(Aq + 4 * (q + 128)), a5 = ld_a4(Aq + 4 * (q + 160));
    const float4 a6 = ld_a4(Aq + 4 * (q + 192)), a7 = ld_a4(Aq + 4 * (q + 224));
    s0 = dot4(a4, *reinterpret_cast<const float4*>(Pq + 4 * (q + 128)), s0);
    s1 = dot4(a5, *reinterpret_cast<const float4*>(Pq + 4 * (q + 160)), s1);
    s2 = dot4(a6, *reinterpret_cast<const float4*>(Pq + 4 * (q + 192)), s2);
    s3 = dot4(a7, *reinterpret_cast<const float4*>(Pq + 4 * (q + 224)), s3);
    const float4 p0 = *reinterpret_cast<const float4*>(Pq + 4 * q);
    const float4 p1 = *reinterpret_cast<const float4*>(Pq + 4 * (q + 32));
    const float4 p2 = *reinterpret_cast<const float4*>(Pq + 4 * (q + 64));
    const float4 p3 = *reinterpret_cast<const float4*>(Pq + 4 * (q + 96));
    s0 = dot4(a0, p0, s0);
    s1 = dot4(a1, p1, s1);
    s2 = dot4(a2, p2, s2);
    s3 = dot4(a3, p3, s3);
  }
  for (; q + 96 < nq; q += 128) {
    s0 = dot4(ld_a4(Aq + 4 * q), *reinterpret_cast<const float4*>(Pq + 4 * q), s0);
    s1 = dot4(ld_a4(Aq + 4 * (q + 32)), *reinterpret_cast<const float4*>(Pq + 4 * (q + 32)), s1);
    s2 = dot4(ld_a4(Aq + 4 * (q + 64)), *reinterpret_cast<const float4*>(Pq + 4 * (q + 64)), s2);
    s3 = dot4(ld_a4(Aq + 4 * (q + 96)), *reinterpret_cast<const float4*>(Pq + 4 * (q + 96)), s3);
  }
  for (; q < nq; q += 32) s0 = dot4(ld_a4(Aq + 4 * q), *reinterpret_cast<const float4*>(Pq + 4 * q), s0);
  if (lane < j0) s1 = fmaf(Ar[lane], P0[lane], s1);
  if (lane < ns - jt) s2 = fmaf(Ar[jt + lane], P0[jt + lane], s2);
  return warp_sum((s0 + s1) + (s2 + s3));
}

// Build the active list and its cost prefix (rows * n per system for the matvec, rows for vectors).
__device__ __forceinline__ int d_build(const DenseBatchArgs& a, const DState& m, bool by_cost) {
  __shared__ int s_n;
  __syncthreads();
  if (threadIdx.x == 0) {
    int c = 0;
    long long acc = 0;
    long long* P = m.prefix();
    for (int s = 0; s < a.S; ++s) {
      if (!m.active(s)) continue;
      m.act()[c] = s;
      P[c] = acc;
      const long long ns = a.sizes[s];
      acc += by_cost ? ns * ns : ns;
      ++c;
    }
    P[c] = acc;
    s_n = c;
  }
  __syncthreads();
  const int r = s_n;
  __syncthreads();
  return r;
}

// (list position, row) of the first row whose cost start is >= c
__device__ __forceinline__ void d_locate(const DenseBatchArgs& a, const DState& m, int nact, long long c, bool by_cost,
                                         int& k, int& row) {
  const long long* P = m.prefix();
  int lo = 0, hi = nact;  // largest k with P[k] <= c
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (P[mid] <= c) lo = mid;
    else hi = mid;
  }
  k = lo;
  const long long ns = a.sizes[m.act()[k]];
  const long long unit = by_cost ? ns : 1;
  long long rr = (c - P[k] + unit - 1) / unit;
  if (rr >= ns) {
    k += 1;
    rr = 0;
  }
  row = (int)rr;
}

// Iterate this warp's share of the active rows: f(s, row, lane) per (system, row) for the matvec
// (whole warp per row), or g(s, row) per lane for elementwise work.  flush(s) at system changes.
template <class RowFn, class Flush>
__device__ __forceinline__ void d_warp_rows(const DenseBatchArgs& a, const DState& m, int nact, bool by_cost, RowFn f,
                                            Flush flush) {
  if (nact == 0) return;
  const long long T = m.prefix()[nact];
  const int W = gridDim.x * (kDBThreads / 32);
  const int w = blockIdx.x * (kDBThreads / 32) + (threadIdx.x >> 5);
  int k0, r0, k1, r1;
  d_locate(a, m, nact, T * w / W, by_cost, k0, r0);
  d_locate(a, m, nact, T * (w + 1) / W, by_cost, k1, r1);
  int k = k0, row = r0;
  while (k < k1 || (k == k1 && row < r1)) {
    if (k >= nact) break;
    const int s = m.act()[k];
    const int ns = a.sizes[s];
    const int end = (k == k1) ? r1 : ns;
    f(s, row, end);
    flush(s);
    k += 1;
    row = 0;
  }
}

// The matvec's rows in chunks of about kDBChunk matrix elements, claimed from a counter in order, so
// that warps whose loads return sooner (SMs nearer the data, less contended) take more chunks and all
// finish together at the grid barrier.  A chunk holds the rows whose cost starts fall inside it.
// Each warp claims its next chunk before working on the current one, hiding the atomic's latency.
// f(s, r0, r1) per (system, row range); flush(s) when the warp moves on to another system and at the
// end.
template <class RowFn, class Flush>
__device__ __forceinline__ void d_claim_rows(const DenseBatchArgs& a, const DState& m, int nact, RowFn f,
                                             Flush flush) {
  if (nact == 0) return;
  const int lane = threadIdx.x & 31;
  const long long T = m.prefix()[nact];
  const long long nch = (T + kDBChunk - 1) / kDBChunk;
  unsigned long long c = 0;
  if (lane == 0) c = atomicAdd(a.claim, 1ull);
  c = __shfl_sync(0xffffffffu, c, 0);
  int last = -1;
  while ((long long)c < nch) {
    unsigned long long next = 0;
    if (lane == 0) next = atomicAdd(a.claim, 1ull);
    int k0, r0, k1, r1;
    d_locate(a, m, nact, (long long)c * kDBChunk, true, k0, r0);
    const long long e = ((long long)c + 1) * kDBChunk;
    d_locate(a, m, nact, e < T ? e : T, true, k1, r1);
    int k = k0, row = r0;
    while (k < k1 || (k == k1 && row < r1)) {
      if (k >= nact) break;
      const int s = m.act()[k];
      const int end = (k == k1) ? r1 : a.sizes[s];
      if (s != last && last >= 0) flush(last);
      last = s;
      f(s, row, end);
      k += 1;
      row = 0;
    }
    c = __shfl_sync(0xffffffffu, next, 0);
  }
  if (last >= 0) flush(last);
}

__global__ void __launch_bounds__(kDBThreads, 4) k_dense_batched_cg(const __grid_constant__ DenseBatchArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  DState m{smem_raw, a.S};
  const int lane = threadIdx.x & 31;
  const int S = a.S;
  double* acc_pap = a.acc;
  double* acc_rr = a.acc + S;
  double* acc_bb = a.acc + 2 * S;

  for (int s = threadIdx.x; s < S; s += blockDim.x) {
    m.active(s) = a.sizes[s] > 0;
    m.it(s) = 0;
  }
  if (threadIdx.x == 0) {
    long long off = 0;
    for (int s = 0; s < S; ++s) {
      m.pbase()[s] = off;
      off += 4 * pcopy_len(a.sizes[s]);
    }
  }
  // |b|^2 (elementwise partition by rows)
  int nact = d_build(a, m, false);
  {
    double part = 0.0;
    d_warp_rows(a, m, nact, false,
                [&](int s, int r0, int r1) {
                  const float* b = a.B + a.v_off[s];
                  for (int i = r0 + lane; i < r1; i += 32) part += (double)b[i] * (double)b[i];
                },
                [&](int s) {
                  const double v = warp_sum(part);
                  if (lane == 0 && v != 0.0) atomicAdd(acc_bb + s, v);
                  part = 0.0;
                });
  }
  if (!grid_sync(a.gb)) return;
  for (int s = threadIdx.x; s < S; s += blockDim.x) m.mult(s) = sqrt(__ldcg(acc_bb + s));
  __syncthreads();
  // r = b / |b| (x0 = 0), p = r, x = 0, |r|^2
  {
    double part = 0.0;
    d_warp_rows(a, m, nact, false,
                [&](int s, int r0, int r1) {
                  const int64_t o = a.v_off[s];
                  const double mu = m.mult(s);
                  float* P0 = a.p4 + m.pbase()[s];
                  const int64_t cs = pcopy_len(a.sizes[s]);
                  for (int i = r0 + lane; i < r1; i += 32) {
                    const float rv = (mu < 1e-40) ? a.B[o + i] / 1e-40f : (float)(a.B[o + i] / mu);
                    a.r[o + i] = rv;
                    put_p(P0, cs, i, rv);
                    a.X[o + i] = 0.f;
                    part += (double)rv * rv;
                  }
                },
                [&](int s) {
                  const double v = warp_sum(part);
                  if (lane == 0 && v != 0.0) atomicAdd(acc_rr + s, v);
                  part = 0.0;
                });
  }
  if (!grid_sync(a.gb)) return;
  for (int s = threadIdx.x; s < S; s += blockDim.x) {
    if (!m.active(s)) continue;
    const double rr = __ldcg(acc_rr + s);
    m.gamma(s) = rr;
    const float rn = (float)sqrt(rr);
    m.rn(s) = rn;
    m.tol_eff(s) = (float)a.tol * rn + (float)a.tol;
    m.active(s) = (rn > m.tol_eff(s)) && a.max_iters > 0;
  }
  __syncthreads();
  if (!grid_sync(a.gb)) return;
  if (blockIdx.x == 0)
    for (int s = threadIdx.x; s < S; s += blockDim.x) acc_rr[s] = 0.0;
  if (!grid_sync(a.gb)) return;

  nact = d_build(a, m, true);
  while (nact > 0) {
    // A: Ap = A p (warp per row), <p, Ap>
    {
      double part = 0.0;
      d_claim_rows(a, m, nact,
                  [&](int s, int r0, int r1) {
                    const int ns = a.sizes[s];
                    const float* A = a.vals + a.a_off[s];
                    const float* P0 = a.p4 + m.pbase()[s];
                    const int64_t cs = pcopy_len(ns);
                    for (int row = r0; row < r1; ++row) {
                      const float v = row_dot(A + (int64_t)row * ns, P0, cs, ns, lane);
                      if (lane == 0) {
                        a.ap[a.v_off[s] + row] = v;
                        part += (double)P0[row] * v;
                      }
                    }
                  },
                  [&](int s) {
                    if (lane == 0 && part != 0.0) atomicAdd(acc_pap + s, part);
                    part = 0.0;
                  });
    }
    if (!grid_sync(a.gb)) return;
    if (blockIdx.x == 0 && threadIdx.x == 0) *a.claim = 0ull;  // next used after two more grid barriers
    for (int j = threadIdx.x; j < nact; j += blockDim.x) {
      const int s = m.act()[j];
      const double pap = __ldcg(acc_pap + s);
      const double den = fabs(pap) < 1e-40 ? 1e-40 : pap;
      const bool conv = m.rn(s) < 1e-40f;
      m.conv(s) = conv ? 1.f : 0.f;
      m.alpha(s) = conv ? 0.f : (float)(m.gamma(s) / den);
    }
    __syncthreads();
    // B: x += alpha p, r -= alpha Ap, |r|^2
    {
      double part = 0.0;
      const int nrow = d_build(a, m, false);
      d_warp_rows(a, m, nrow, false,
                  [&](int s, int r0, int r1) {
                    const int64_t o = a.v_off[s];
                    const float al = m.alpha(s);
                    const float* P0 = a.p4 + m.pbase()[s];
                    for (int i = r0 + lane; i < r1; i += 32) {
                      a.X[o + i] += al * P0[i];
                      const float rv = a.r[o + i] - al * a.ap[o + i];
                      a.r[o + i] = rv;
                      part += (double)rv * rv;
                    }
                  },
                  [&](int s) {
                    const double v = warp_sum(part);
                    if (lane == 0 && v != 0.0) atomicAdd(acc_rr + s, v);
                    part = 0.0;
                  });
    }
    if (!grid_sync(a.gb)) return;
    if (blockIdx.x == 0)
      for (int s = threadIdx.x; s < S; s += blockDim.x) acc_pap[s] = 0.0;
    for (int j = threadIdx.x; j < nact; j += blockDim.x) {
      const int s = m.act()[j];
      const double g1 = __ldcg(acc_rr + s);
      const double den = fabs(m.gamma(s)) < 1e-40 ? 1e-40 : m.gamma(s);
      m.beta(s) = m.conv(s) != 0.f ? 0.f : (float)(g1 / den);
      m.gamma(s) = g1;
      const float rn = (float)sqrt(g1);
      m.rn(s) = rn;
      m.it(s) += 1;
      m.active(s) = (rn > m.tol_eff(s)) && (m.it(s) < a.max_iters);
    }
    __syncthreads();
    if (!grid_sync(a.gb)) return;  // everyone has read acc_rr
    if (blockIdx.x == 0)
      for (int s = threadIdx.x; s < S; s += blockDim.x) acc_rr[s] = 0.0;
    // C: p = r + beta p (systems that go on)
    const int nrow = d_build(a, m, false);
    d_warp_rows(a, m, nrow, false,
                [&](int s, int r0, int r1) {
                  const int64_t o = a.v_off[s];
                  const float b = m.beta(s);
                  float* P0 = a.p4 + m.pbase()[s];
                  const int64_t cs = pcopy_len(a.sizes[s]);
                  for (int i = r0 + lane; i < r1; i += 32) put_p(P0, cs, i, a.r[o + i] + b * P0[i]);
                },
                [&](int) {});
    if (!grid_sync(a.gb)) return;
    nact = d_build(a, m, true);
  }
  // x *= |b|
  for (int s = threadIdx.x; s < S; s += blockDim.x) m.active(s) = a.sizes[s] > 0;
  nact = d_build(a, m, false);
  d_warp_rows(a, m, nact, false,
              [&](int s, int r0, int r1) {
                const int64_t o = a.v_off[s];
                const float mu = (float)m.mult(s);
                for (int i = r0 + lane; i < r1; i += 32) a.X[o + i] *= mu;
              },
              [&](int) {});
  if (blockIdx.x == 0)
    for (int s = threadIdx.x; s < S; s += blockDim.x) {
      if (a.out_iters) a.out_iters[s] = m.it(s);
      if (a.out_status) a.out_status[s] = (m.rn(s) > m.tol_eff(s)) ? COLAGB_SYS_MAX_ITERS : COLAGB_SYS_CONVERGED;
    }
}

}  // namespace colagb

using namespace colagb;

extern "C" int colagb_cg_dense_batched_workspace_bytes(int64_t num_systems, int64_t total_rows, size_t* bytes) {
  if (!bytes || num_systems < 0 || total_rows < 0) return fail(COLAGB_ERR_INVALID, "dense batched CG: bad arguments");
  Bump ws = Bump::measuring();
  ws.take<float>(total_rows);
  ws.take<float>(4 * (total_rows + 8 * num_systems));  // >= 4 * sum of pcopy_len(n_s)
  ws.take<float>(total_rows);
  ws.take<double>(3 * (num_systems > 0 ? num_systems : 1));
  ws.take<unsigned int>(8);
  ws.take<unsigned long long>(1);
  *bytes = ws.peak;
  return COLAGB_OK;
}

extern "C" int colagb_cg_dense_batched_solve(int64_t num_systems, const int32_t* sizes, const int64_t* a_offsets,
                                             const int64_t* v_offsets, int64_t total_rows, const float* values,
                                             const float* B, float* X, double tol, int32_t max_iters,
                                             int32_t* per_system_iters, int32_t* per_system_status, void* workspace,
                                             size_t workspace_bytes, void* stream) {
  if (num_systems < 0 || num_systems > kDBMaxSystems || total_rows < 0 || max_iters < 0)
    return fail(COLAGB_ERR_INVALID, "dense batched CG: need 0 <= num_systems <= 1024, max_iters >= 0");
  if (num_systems == 0 || total_rows == 0) return COLAGB_OK;
  if (!sizes || !a_offsets || !v_offsets || !values || !B || !X)
    return fail(COLAGB_ERR_INVALID, "dense batched CG: null argument");
  size_t need = 0;
  COLAGB_TRY(colagb_cg_dense_batched_workspace_bytes(num_systems, total_rows, &need));
  if (!workspace || workspace_bytes < need) return fail(COLAGB_ERR_WORKSPACE, "dense batched CG: workspace too small");
  Bump ws(workspace, workspace_bytes);
  DenseBatchArgs a;
  a.S = (int)num_systems;
  a.sizes = sizes;
  a.a_off = a_offsets;
  a.v_off = v_offsets;
  a.vals = values;
  a.B = B;
  a.X = X;
  a.r = ws.take<float>(total_rows);
  a.p4 = ws.take<float>(4 * (total_rows + 8 * num_systems));
  a.ap = ws.take<float>(total_rows);
  a.acc = ws.take<double>(3 * num_systems);
  unsigned int* bar = ws.take<unsigned int>(8);
  a.claim = ws.take<unsigned long long>(1);
  a.out_iters = per_system_iters;
  a.out_status = per_system_status;
  a.tol = tol;
  a.max_iters = max_iters;
  a.gb.count = bar;
  a.gb.generation = bar + 1;
  a.gb.err = reinterpret_cast<int*>(bar + 2);
  a.gb.spin_limit = kDefaultSpinLimit;
  cudaStream_t st = as_stream(stream);
  const size_t smem = dense_batch_smem(a.S);
  if (smem > 48 * 1024)
    COLAGB_CUDA(cudaFuncSetAttribute(k_dense_batched_cg, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int occ = 0;
  COLAGB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_dense_batched_cg, kDBThreads, smem));
  if (occ < 1) return fail(COLAGB_ERR_UNSUPPORTED, "dense batched CG kernel cannot be resident");
  const int nb = num_sms() * (occ < 4 ? occ : 4);
  a.gb.nblocks = (unsigned)nb;
  COLAGB_CUDA(cudaMemsetAsync(bar, 0, 8 * sizeof(unsigned int), st));
  COLAGB_CUDA(cudaMemsetAsync(a.claim, 0, sizeof(unsigned long long), st));
  COLAGB_CUDA(cudaMemsetAsync(a.acc, 0, 3 * num_systems * sizeof(double), st));
  void* args[] = {&a};
  COLAGB_CUDA(cudaLaunchCooperativeKernel((const void*)k_dense_batched_cg, dim3(nb), dim3(kDBThreads), args, smem, st));
  unsigned int herr = 0;
  COLAGB_CUDA(cudaMemcpyAsync(&herr, bar + 2, sizeof(unsigned int), cudaMemcpyDeviceToHost, st));
  COLAGB_CUDA(cudaStreamSynchronize(st));
  if (herr != 0) return fail(COLAGB_ERR_TIMEOUT, "dense batched CG: a grid barrier timed out");
  return COLAGB_OK;
}

// ---------------------------------------------------------------------------------------------
// FP64 residual of the uneven dense batch, for iterative refinement on top of the FP32 CG above:
// R = B - A X in FP64 (A's FP32 values, FP64 products and sums), one warp per row, plus |r_s|^2 per
// system.  The system of a row comes from a binary search of v_offsets.

namespace colagb {

__global__ void __launch_bounds__(256) k_dense_residual64(int S, const int32_t* __restrict__ sizes,
                                                          const int64_t* __restrict__ a_off,
                                                          const int64_t* __restrict__ v_off, int64_t total_rows,
                                                          const float* __restrict__ vals,
                                                          const double* __restrict__ B, const double* __restrict__ X,
                                                          double* __restrict__ R, double* __restrict__ rr) {
  const int lane = threadIdx.x & 31;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t g = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; g < total_rows; g += nwarps) {
    int lo = 0, hi = S - 1;  // last system whose v_off <= g
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (v_off[mid] <= g) lo = mid;
      else hi = mid - 1;
    }
    const int s = lo;
    const int64_t n = sizes[s];
    const int64_t i = g - v_off[s];
    const float* row = vals + a_off[s] + i * n;
    const double* x = X + v_off[s];
    double acc = 0.0;
    for (int64_t j = lane; j < n; j += 32) acc += (double)row[j] * x[j];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) {
      const double r = B[g] - acc;
      R[g] = r;
      atomicAdd(rr + s, r * r);
    }
  }
}

}  // namespace colagb

extern "C" int colagb_dense_batched_residual64(int64_t num_systems, const int32_t* sizes, const int64_t* a_offsets,
                                               const int64_t* v_offsets, int64_t total_rows, const float* values,
                                               const double* B, const double* X, double* R, double* rr,
                                               void* stream) {
  if (num_systems < 1 || num_systems > kDBMaxSystems || total_rows < 0 || !sizes || !a_offsets || !v_offsets ||
      !values || !B || !X || !R || !rr)
    return fail(COLAGB_ERR_INVALID, "colagb_dense_batched_residual64: bad arguments");
  cudaStream_t st = as_stream(stream);
  COLAGB_CUDA(cudaMemsetAsync(rr, 0, num_systems * sizeof(double), st));
  if (total_rows == 0) return COLAGB_OK;
  const int64_t want = ceil_div(total_rows * 32, 256);
  const int blocks = (int)std::min<int64_t>(want, (int64_t)num_sms() * 16);
  k_dense_residual64<<<blocks, 256, 0, st>>>((int)num_systems, sizes, a_offsets, v_offsets, total_rows, values, B, X,
                                             R, rr);
  COLAGB_CUDA(cudaGetLastError());
  return COLAGB_OK;
}
