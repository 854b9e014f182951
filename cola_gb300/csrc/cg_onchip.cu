// Batched shared-pattern PCG with the Krylov vectors held on chip: one thread-block cluster per
// system, the system's p, r and FP32 solution correction d spread over the shared memory of the
// cluster's CTAs, the matrix streamed from diagonal storage.
//
// Same algorithm and stop rule as the other batched schedules (cg_batched.cu, cg_cluster.cu: FP32
// PCG, FP64 solution, FP64 residual replacement, Jacobi / FSAI, the FP64 true residual as the only
// convergence test and as the judge of a learned FSAI factor).  What changes is where data lives:
//   * a pattern made of a few constant-offset diagonals (any stencil on a structured grid) is
//     stored as diagonals: values[k][i] = A(i, i + off[k]), one coalesced stream per diagonal, no
//     column indices, no row pointers;
//   * CTA `rank` of the cluster owns rows [rank * R, rank * R + R); its p and r (plus a halo of H
//     rows on each side) and d live in its shared memory for the whole solve, so the only memory
//     traffic per iteration is the matrix (and the FSAI operator M = G^T G, also diagonal, in
//     bfloat16);
//   * each CTA stores its edge rows straight into the neighbouring CTAs' halos (distributed shared
//     memory) before the cluster barrier that publishes them, and its reduction partials into every
//     peer, so nothing is loaded from a peer on the critical path;
//   * per-row values that stay with the same thread between phases (A p, then z) stay in registers;
//   * clusters are persistent: each takes the next system from an atomic counter, converts that
//     system's CSR values into its own diagonal slot, solves it and moves on.
// Results are per system and independent of the scheduling order.
#include <cooperative_groups.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <mutex>
#include <string>
#include <type_traits>
#include <vector>

#include "cluster.cuh"
#include "common.cuh"

namespace cg = cooperative_groups;

namespace colagb {

constexpr int kOT = 512;         // threads per CTA
constexpr int kRowBatch = 8;     // rows per thread whose loads are issued together in the FP64 passes
constexpr int kMaxDiagA = 9;     // diagonals of A
constexpr int kMaxDiagG = 5;     // diagonals of the FSAI factor G
constexpr int kMaxDiagM = 17;    // diagonals of M = G^T G
constexpr int kMaxPairs = 32;    // (G diagonal, G diagonal) products that make up M
constexpr size_t kOnchipSmemMax = 227 * 1024 - 1024;
// The FSAI operator M = G^T G is stored in bfloat16 (round to nearest: each entry off by at most
// 2^-8 of itself) with every main-diagonal entry raised by kMBoost = 2^-7 times its row's absolute
// sum.  The change to M is then diagonally dominant with a non-negative diagonal, so the stored M'
// satisfies M' >= M > 0 (Gershgorin): still SPD and symmetric, a preconditioner within ~1 % of M,
// at half the bytes per step.  A stays FP32 (CG's operator), and the FP64 true residual still judges
// convergence.
constexpr float kMBoost = 1.f / 128.f;

struct OnchipArgs {
  int64_t n, S, np;  // rows, systems, rows padded to the cluster (CL * R)
  int R, H;          // rows per CTA, halo rows on each side
  int nd, center;    // diagonals of A and the index of offset 0 (-1: no main diagonal)
  int off[kMaxDiagA];
  int ng, nm;
  int goff[kMaxDiagG];
  int moff[kMaxDiagM];
  int pstart[kMaxDiagM + 1];
  int pa[kMaxPairs], pb[kMaxPairs];  // M(i, i + moff[m]) = sum G(k, i) G(k, i + moff[m]), k = i - goff[pa]
  const int32_t* indptr;
  const int32_t* indices;
  const float* vals;
  int64_t vstride;
  const int32_t* g_indptr;
  const int32_t* g_indices;
  const float* g_vals;
  int64_t g_nnz;
  float* adia;  // [slot][nd][np]
  float* gdia;  // [slot][ng][np]
  float* mdia;  // [slot][nm][np] floats of space, holding bfloat16 diagonals [slot][nm][np]
  float* dinv;  // [slot][np]: 1 / A(i, i) (1 where the diagonal is absent or zero)
  unsigned int* next;
  const double* B;
  double* X;
  int* out_status;
  int* out_iters;
  double* out_relres;
  int* out_nrep;
  double tol, inner_tol;
  int max_sweeps, max_inner, prec_kind, fallback, mode;
};

// One CSR row as dense values on diagonal `o` (entries with the same column are summed).
__device__ __forceinline__ float csr_diag_value(const int32_t* indptr, const int32_t* indices, const float* vals,
                                                int64_t i, int o) {
  float v = 0.f;
  for (int32_t e = indptr[i]; e < indptr[i + 1]; ++e)
    if ((int64_t)indices[e] - i == o) v += vals[e];
  return v;
}

// Row i of a CSR matrix into diagonal storage: out[k * stride] = the sum, in CSR order, of the
// row's entries in column i + off[k], for k < nk (0 for a row past n).  A row of at most eight
// entries is loaded once, all loads in flight together, and matched against every diagonal from
// registers; a longer row is scanned once per diagonal.
__device__ __forceinline__ void csr_row_to_diagonals(const int32_t* indptr, const int32_t* indices, const float* vals,
                                                     int64_t i, bool live, const int* off, int nk, float* out,
                                                     int64_t stride) {
  const int32_t b = live ? indptr[i] : 0, e = live ? indptr[i + 1] : 0;
  if (e - b <= 8) {
    int32_t col[8];
    float v[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const bool ok = b + u < e;
      col[u] = ok ? indices[b + u] : 0;
      v[u] = ok ? vals[b + u] : 0.f;
    }
#pragma unroll 1
    for (int k = 0; k < nk; ++k) {
      const int64_t c = i + off[k];
      float acc = 0.f;
#pragma unroll
      for (int u = 0; u < 8; ++u)
        if (b + u < e && col[u] == c) acc += v[u];
      out[k * stride] = acc;
    }
  } else {
#pragma unroll 1
    for (int k = 0; k < nk; ++k) out[k * stride] = csr_diag_value(indptr, indices, vals, i, off[k]);
  }
}

// Per-CTA geometry of the on-chip schedule.
struct OnchipCta {
  int rank, R, H, tid;
  int64_t np, i0;  // padded rows per diagonal, first row of this CTA
};

// Thread `tid` owns the float4s q = tid + j kOT (j < G4) of its CTA (rows q, q + S, q + 2S, q + 3S
// in the strip layout below): every load and store of the hot loops is 128 bits wide and
// consecutive threads touch consecutive 16-byte words (coalesced global accesses, conflict-free
// shared-memory accesses).
__device__ __forceinline__ float4 ld4(const float* p) { return *reinterpret_cast<const float4*>(p); }
__device__ __forceinline__ void st4(float* p, float4 v) { *reinterpret_cast<float4*>(p) = v; }
__device__ __forceinline__ float dot4(float4 a, float4 b) { return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w; }

// Strip layout of the on-chip vectors and diagonals.  A CTA's R own rows are four strips of
// S = R / 4 rows; float4 number q (0 <= q < S) holds rows q, q + S, q + 2S, q + 3S, so a shift of
// the row index by any offset o is a shift of q by o: every operand of a diagonal product is one
// aligned 128-bit load.  Vectors with a halo also hold q in [-H, 0) and [S, S + H): there component
// c is row q + c S, i.e. the adjacent strip of this CTA -- except component 0 of the left halo and
// component 3 of the right one, which are the neighbouring CTAs' edge rows (zero at the ends of the
// cluster).  Local row l sits at float index sidx(l).
__device__ __forceinline__ int sidx(int l, int S) { return 4 * (l % S) + l / S; }

// The halo of v (strip layout): the components from this CTA's adjacent strips, and the neighbouring
// CTAs' edge rows read from their shared memory (after a cluster barrier that published them).
template <int CL>
__device__ __forceinline__ void fill_halo(cg::cluster_group& cl, const OnchipCta& c, float* v) {
  const int S = c.R / 4;
  for (int h = c.tid; h < c.H; h += kOT) {
    const int qe = S - c.H + h;  // left halo index h - H <- the strips' ends
    const float4 e = ld4(v + 4 * qe);
    const float l0 = c.rank > 0 ? *cl.map_shared_rank(v + 4 * qe + 3, c.rank - 1) : 0.f;
    st4(v + 4 * (h - c.H), make_float4(l0, e.x, e.y, e.z));
    const float4 b = ld4(v + 4 * h);  // right halo index S + h <- the strips' starts
    const float r3 = c.rank + 1 < CL ? *cl.map_shared_rank(v + 4 * h, c.rank + 1) : 0.f;
    st4(v + 4 * (S + h), make_float4(b.y, b.z, b.w, r3));
  }
}

// After this thread has written its own float4s of v (strip layout), the halo entries they feed:
//   * strip 0's first H rows (component x of q < H) into the left neighbour's right-halo component 3,
//     strip 3's last H rows (component w of q >= S - H) into the right neighbour's left-halo
//     component 0 -- stores into the neighbours' shared memory, so the reader's halo is complete
//     when the cluster barrier that follows (arrive.release / wait.acquire) returns, with no load on
//     its critical path;
//   * the components of this CTA's own halo that come from its adjacent strips.
// Scalar stores: the neighbour writes the remaining component of the same 16 bytes.  The halos'
// cluster-end components are never written (zero from the system's setup).  A writer only writes
// after the cluster barrier that ends the reader's last use of that halo.  The thread re-reads its
// own just-written float4s (no barrier needed; a pass of its own keeps the phase loops' registers).
template <int CL>
__device__ __forceinline__ void push_edge_lo(cg::cluster_group& cl, const OnchipCta& c, float* v, int S, int q) {
  const float4 x = ld4(v + 4 * q);  // q < H: strip starts
  if (c.rank > 0) *cl.map_shared_rank(v + 4 * (S + q) + 3, c.rank - 1) = x.x;
  float* h = v + 4 * (S + q);  // own right halo, components 0..2
  *reinterpret_cast<float2*>(h) = make_float2(x.y, x.z);
  h[2] = x.w;
}
template <int CL>
__device__ __forceinline__ void push_edge_hi(cg::cluster_group& cl, const OnchipCta& c, float* v, int S, int q) {
  const float4 x = ld4(v + 4 * q);  // q >= S - H: strip ends
  if (c.rank + 1 < CL) *cl.map_shared_rank(v + 4 * (q - S), c.rank + 1) = x.w;
  float* h = v + 4 * (q - S);  // own left halo, components 1..3
  h[1] = x.x;
  *reinterpret_cast<float2*>(h + 2) = make_float2(x.y, x.z);
}
// Phases B and C visit the groups edge-first (0, G4 - 1, 1, 2, ...) and push an edge group as soon
// as it is stored (push_group), so that the stores into the neighbours are in flight while the
// other groups are updated instead of holding up the barrier's release.  When H > kOT the edge
// rows span more groups and push_halos_wide pushes them after the phase.
template <int G4>
__device__ constexpr int edge_first(int t) { return t == 0 ? 0 : (t == 1 ? G4 - 1 : t - 1); }

template <int CL, int G4>
__device__ __forceinline__ void push_group(cg::cluster_group& cl, const OnchipCta& c, float* v, int j) {
  if (c.H > kOT) return;
  const int S = c.R / 4;
  if (j == 0 && c.tid < c.H) push_edge_lo<CL>(cl, c, v, S, c.tid);
  if (j == G4 - 1) {
    const int q = c.tid + (G4 - 1) * kOT;
    if (q >= S - c.H) push_edge_hi<CL>(cl, c, v, S, q);
  }
}

template <int CL, int G4>
__device__ __forceinline__ void push_halos_wide(cg::cluster_group& cl, const OnchipCta& c, float* v) {
  if (c.H <= kOT) return;
  const int S = c.R / 4;
#pragma unroll 1
  for (int j = 0; j < G4; ++j) {
    const int q = c.tid + j * kOT;
    if (q < c.H) push_edge_lo<CL>(cl, c, v, S, q);
    if (q >= S - c.H) push_edge_hi<CL>(cl, c, v, S, q);
  }
}

template <int CL, int G4>
__device__ __forceinline__ void push_halos(cg::cluster_group& cl, const OnchipCta& c, float* v) {
  const int S = c.R / 4;
  if (c.H <= kOT) {  // the edge float4s are this thread's first and last groups only
    if (c.tid < c.H) push_edge_lo<CL>(cl, c, v, S, c.tid);
    const int q = c.tid + (G4 - 1) * kOT;
    if (q >= S - c.H) push_edge_hi<CL>(cl, c, v, S, q);
    return;
  }
#pragma unroll 1
  for (int j = 0; j < G4; ++j) {
    const int q = c.tid + j * kOT;
    if (q < c.H) push_edge_lo<CL>(cl, c, v, S, q);
    if (q >= S - c.H) push_edge_hi<CL>(cl, c, v, S, q);
  }
}

// The four diagonal values of one float4 group as they sit in registers between load and use: FP32
// (A) or bfloat16 (M, 8 bytes per group, widened to FP32 when used).
template <typename T>
struct Diag4;
template <>
struct Diag4<float> {
  using Reg = float4;
  static __device__ __forceinline__ Reg load(const float* p) { return ld4(p); }
  static __device__ __forceinline__ float4 wide(Reg r) { return r; }
};
template <>
struct Diag4<__nv_bfloat16> {
  using Reg = uint2;
  static __device__ __forceinline__ Reg load(const __nv_bfloat16* p) { return *reinterpret_cast<const uint2*>(p); }
  static __device__ __forceinline__ float4 wide(Reg r) {  // bfloat16 = the high half of an FP32 word
    return make_float4(__uint_as_float(r.x << 16), __uint_as_float(r.x & 0xffff0000u), __uint_as_float(r.y << 16),
                       __uint_as_float(r.y & 0xffff0000u));
  }
};

// zq[j] = sum_k D[k][rows of group j] * v[rows + off[k]], k ascending (the host puts the main
// diagonal last, the others in column order); returns this thread's part of <v, D v>.  One
// diagonal at a time over all of the thread's groups (G4 128-bit loads per thread, ~64 KB per SM
// for FP32), pipelined by halves: once the first half of diagonal k has been
// used, its registers load the first half of diagonal k + 1 while the second half of k is still
// arriving.  (Waiting for a whole diagonal before issuing the next cost one L2 round trip plus the
// transfer per diagonal, ~1.9k cycles for 64 KB per SM; double-buffering whole diagonals needs more
// registers than the 128 a thread has here next to the G4 result registers.)  `pending`: a
// cluster_arrive() publishing v's own rows and the halos pushed into the neighbours (push_halos) is
// outstanding; the first diagonal's loads are issued before waiting on it (the matrix does not
// depend on it).
template <int CL, int G4, typename T>
__device__ __forceinline__ float diag_product(cg::cluster_group& cl, const OnchipCta& c, float4 (&zq)[G4],
                                              const T* D, const int* off, int nk, float* v, bool pending) {
  using DL = Diag4<T>;
  typename DL::Reg a4[G4];
  const T* D0 = D + c.i0;
#pragma unroll
  for (int j = 0; j < G4; ++j) a4[j] = DL::load(D0 + 4 * (c.tid + j * kOT));
  if (pending) cluster_wait();  // v's own rows and both halos complete
#pragma unroll
  for (int j = 0; j < G4; ++j) zq[j] = make_float4(0.f, 0.f, 0.f, 0.f);
  float dotv = 0.f;
  for (int k = 0; k < nk; ++k) {
    const int o = off[k];
    const bool more = k + 1 < nk;  // the same for every thread
    const T* Dn = D + (k + 1) * c.np + c.i0;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      // the shared-memory operands in two halves, so at most half of them are held at once
      float4 pv[G4 / 2];
#pragma unroll
      for (int jj = 0; jj < G4 / 2; ++jj) pv[jj] = ld4(v + 4 * (c.tid + (h * (G4 / 2) + jj) * kOT + o));
#pragma unroll
      for (int jj = 0; jj < G4 / 2; ++jj) {
        const int j = h * (G4 / 2) + jj;
        const float4 av = DL::wide(a4[j]);
        zq[j].x = fmaf(av.x, pv[jj].x, zq[j].x);
        zq[j].y = fmaf(av.y, pv[jj].y, zq[j].y);
        zq[j].z = fmaf(av.z, pv[jj].z, zq[j].z);
        zq[j].w = fmaf(av.w, pv[jj].w, zq[j].w);
      }
      if (!more && o == 0) {  // the last diagonal is the main one: pv holds v's own rows
#pragma unroll
        for (int jj = 0; jj < G4 / 2; ++jj) dotv += dot4(pv[jj], zq[h * (G4 / 2) + jj]);
      }
      // this half's registers are free: they take the same half of the next diagonal, so the other
      // half's loads are still in flight when these are issued (the stream never drains between
      // diagonals, and no register is added)
      if (more) {
#pragma unroll
        for (int jj = 0; jj < G4 / 2; ++jj) {
          const int j = h * (G4 / 2) + jj;
          a4[j] = DL::load(Dn + 4 * (c.tid + j * kOT));
        }
      }
    }
  }
  if (off[nk - 1] != 0) {  // no main diagonal: read v's own rows again
#pragma unroll
    for (int j = 0; j < G4; ++j) dotv += dot4(ld4(v + 4 * (c.tid + j * kOT)), zq[j]);
  }
  return dotv;
}

// z = M r into zq, returns this thread's part of <r, z>.  The per-iteration inner products are FP32
// like the vectors (FP64 arithmetic runs at 1/64 of the FP32 rate on this GPU and would sit on the
// critical path of every step); FP64 is kept for |b|, the true residual that judges convergence, and
// x.  FSAI: `published` says a cluster_arrive() publishing r's own rows is outstanding.
template <int CL, int G4>
__device__ __forceinline__ float apply_z(cg::cluster_group& cl, const OnchipCta& c, float4 (&zq)[G4], int prec,
                                         const OnchipArgs& a, const __nv_bfloat16* M, const float* Dv, float* rs,
                                         bool published) {
  if (prec == COLAGB_PREC_FSAI) return diag_product<CL, G4, __nv_bfloat16>(cl, c, zq, M, a.moff, a.nm, rs, published);
  if (prec == COLAGB_PREC_JACOBI) {
#pragma unroll
    for (int j = 0; j < G4; ++j) {
      const int l = 4 * (c.tid + j * kOT);
      const float4 d = ld4(Dv + c.i0 + l), r = ld4(rs + l);
      zq[j] = make_float4(d.x * r.x, d.y * r.y, d.z * r.z, d.w * r.w);
    }
  } else {
#pragma unroll
    for (int j = 0; j < G4; ++j) zq[j] = ld4(rs + 4 * (c.tid + j * kOT));
  }
  float rz = 0.f;
#pragma unroll
  for (int j = 0; j < G4; ++j) rz += dot4(ld4(rs + 4 * (c.tid + j * kOT)), zq[j]);
  return rz;
}

// Data written inside this kernel by other CTAs (the G diagonals, X) is read with plain loads after
// a cluster barrier; nothing written here is read through the non-coherent read-only path.
template <int CL, int G>
__global__ void __launch_bounds__(kOT, 1) k_onchip_pcg(const __grid_constant__ OnchipArgs a) {
  cg::cluster_group cl = cg::this_cluster();
  const int rank = (int)cl.block_rank();
  const int64_t slot = blockIdx.x / CL;
  extern __shared__ __align__(16) float smem[];
  __shared__ double slots[2][8];
  __shared__ double red[32];
  __shared__ double bcast[8];
  __shared__ float fslots[2][2 * CL];  // cluster_sum_f slots: NQ <= 2 sums x CL ranks
  __shared__ float wpart[2 * 32];
  __shared__ unsigned int s_sys;
  int buf = 0, fbuf = 0;
  auto next_slot = [&]() { double* q = slots[buf]; buf ^= 1; return q; };
  auto next_fslot = [&]() { float* q = fslots[fbuf]; fbuf ^= 1; return q; };

  const int R = a.R, H = a.H;
  const int64_t n = a.n, np = a.np;
  const int S = R / 4;                     // strip length (strip layout, see sidx)
  float* ps = smem + 4 * H;                // p: float4 indices [-H, S + H)
  float* rs = smem + (R + 8 * H) + 4 * H;  // r: float4 indices [-H, S + H)
  float* ds = smem + 2 * (R + 8 * H);      // d: float4 indices [0, S)
  const int tid = threadIdx.x;
  const int64_t i0 = (int64_t)rank * R;  // first row of this CTA (rows >= n are zero padding)
  float* A = a.adia + slot * a.nd * np;
  float* Gd = a.gdia ? a.gdia + slot * a.ng * np : nullptr;
  __nv_bfloat16* M = a.mdia ? reinterpret_cast<__nv_bfloat16*>(a.mdia + slot * a.nm * np) : nullptr;
  float* Dv = a.dinv + slot * np;
  const OnchipCta ctx{rank, R, H, tid, np, i0};
  constexpr int G4 = G / 4;  // 4-row groups per thread

  while (true) {
    if (rank == 0 && tid == 0) s_sys = atomicAdd(a.next, 1u);
    cl.sync();
    const int64_t s = *cl.map_shared_rank(&s_sys, 0);
    cl.sync();  // every CTA has read the system index before rank 0 may replace it or leave
    if (s >= a.S) break;

    const float* vals = a.vals + s * a.vstride;
    const double* B = a.B + s * n;
    double* X = a.X + s * n;
    int prec = a.prec_kind;

    // ---- setup: diagonal slots, x = 0, on-chip vectors zero, |b|^2 ----
    double v1[1] = {0.0};
#pragma unroll 1
    for (int l = tid; l < R; l += kOT) {
      const int64_t i = i0 + l;
      const bool live = i < n;
      const int64_t si = i0 + sidx(l, S);  // this row's place in the diagonal slots
      csr_row_to_diagonals(a.indptr, a.indices, vals, i, live, a.off, a.nd, A + si, np);
      Dv[si] = a.center >= 0 && A[a.center * np + si] != 0.f ? 1.f / A[a.center * np + si] : 1.f;
      if (Gd) csr_row_to_diagonals(a.g_indptr, a.g_indices, a.g_vals + s * a.g_nnz, i, live, a.goff, a.ng, Gd + i, np);
      ps[l] = 0.f;
      rs[l] = 0.f;
      ds[l] = 0.f;
      if (l < 4 * H) {  // halos (their components at the ends of the cluster stay zero)
        ps[l - 4 * H] = 0.f;
        ps[R + l] = 0.f;
        rs[l - 4 * H] = 0.f;
        rs[R + l] = 0.f;
      }
      if (live) {
        const double bv = B[i];
        v1[0] += bv * bv;
        X[i] = 0.0;
      }
    }
    cluster_sum<1, CL>(cl, v1, next_slot(), red, bcast);  // also publishes G's diagonals and x = 0
    if (M) {  // M = G^T G on this CTA's rows, from G's diagonals (rows k >= i may belong to the next CTA)
#pragma unroll 1
      for (int l0 = tid; l0 < R; l0 += kRowBatch * kOT) {  // eight rows' loads in flight per product
        float asum[kRowBatch], ctr[kRowBatch];  // row absolute sums, main-diagonal values
#pragma unroll
        for (int u = 0; u < kRowBatch; ++u) asum[u] = ctr[u] = 0.f;
        int mc = 0;
#pragma unroll 1
        for (int m = 0; m < a.nm; ++m) {
          float v[kRowBatch];
#pragma unroll
          for (int u = 0; u < kRowBatch; ++u) v[u] = 0.f;
#pragma unroll 1
          for (int q = a.pstart[m]; q < a.pstart[m + 1]; ++q) {
            const float* ga = Gd + a.pa[q] * np;
            const float* gb = Gd + a.pb[q] * np;
            const int go = a.goff[a.pa[q]];
#pragma unroll
            for (int u = 0; u < kRowBatch; ++u) {
              const int64_t i = i0 + l0 + u * kOT;
              const int64_t k = i - go;  // go <= 0: k >= i
              if (i < n && k < n) v[u] += ga[k] * gb[k];
            }
          }
#pragma unroll
          for (int u = 0; u < kRowBatch; ++u) asum[u] += fabsf(v[u]);
          if (a.moff[m] == 0) {
            mc = m;
#pragma unroll
            for (int u = 0; u < kRowBatch; ++u) ctr[u] = v[u];
          } else {
#pragma unroll
            for (int u = 0; u < kRowBatch; ++u) M[m * np + i0 + sidx(l0 + u * kOT, S)] = __float2bfloat16_rn(v[u]);
          }
        }
#pragma unroll
        for (int u = 0; u < kRowBatch; ++u)
          M[mc * np + i0 + sidx(l0 + u * kOT, S)] = __float2bfloat16_rn(ctr[u] + kMBoost * asum[u]);
      }
    }
    const double bnorm = sqrt(v1[0]);
    int status = COLAGB_SYS_RUNNING;
    double relres = bnorm > 0.0 ? 1.0 : 0.0;
    if (!(bnorm > 0.0)) status = bnorm == 0.0 ? COLAGB_SYS_CONVERGED : COLAGB_SYS_NAN;
    const double binv = bnorm > 0.0 ? 1.0 / bnorm : 1.0;

    // r = b/|b| - A x in FP64 (x gathered from global memory), |r|^2
    float4 zq[G4];  // per-row register values: A p in phase A, z in phases B/C
    // Eight rows per thread per pass, diagonal by diagonal: the eight rows' loads of one diagonal are
    // in flight together (a row at a time paid one L2 round trip per term).  Terms are added in
    // diagonal order, as in the CSR row.
    auto residual = [&](double& rr) {
      rr = 0.0;
#pragma unroll 1
      for (int l0 = tid; l0 < R; l0 += kRowBatch * kOT) {  // R is a multiple of kRowBatch * kOT
        double ax[kRowBatch];
#pragma unroll
        for (int u = 0; u < kRowBatch; ++u) ax[u] = 0.0;
#pragma unroll 1
        for (int k = 0; k < a.nd; ++k) {
          const float* Ak = A + k * np + i0;
          const int o = a.off[k];
#pragma unroll
          for (int u = 0; u < kRowBatch; ++u) {
            const int l = l0 + u * kOT;
            const int64_t c = i0 + l + o;
            const float av = Ak[sidx(l, S)];  // 0 where row i0 + l has no entry on this diagonal (and past n)
            const double xv = c >= 0 && c < n ? X[c] : 0.0;
            ax[u] += (double)av * xv;
          }
        }
#pragma unroll
        for (int u = 0; u < kRowBatch; ++u) {
          const int l = l0 + u * kOT;
          const int64_t i = i0 + l;
          if (i < n) {
            const double rv = B[i] * binv - ax[u];
            rs[sidx(l, S)] = (float)rv;
            rr += rv * rv;
          }
        }
      }
    };
    double q2[1];
    residual(q2[0]);
    cluster_sum<1, CL>(cl, q2, next_slot(), red, bcast);
    float rn = (float)sqrt(q2[0]);
    float rmax = rn;
    double relres_prev = relres;
    if (prec == COLAGB_PREC_FSAI) fill_halo<CL>(cl, ctx, rs);
    __syncthreads();
    float q1[1] = {apply_z<CL, G4>(cl, ctx, zq, prec, a, M, Dv, rs, false)};
    cluster_sum_f<1, CL>(cl, q1, wpart, next_fslot());
    float gamma = q1[0];
    if (status == COLAGB_SYS_RUNNING && rn <= (float)a.tol) status = COLAGB_SYS_CONVERGED;
#pragma unroll
    for (int j = 0; j < G4; ++j) st4(ps + 4 * (tid + j * kOT), zq[j]);
    push_halos<CL, G4>(cl, ctx, ps);
    __syncthreads();
    cluster_arrive();  // p and its halos published; waited for inside the first step
    bool arrived = true;

    int it = 0, nrep = 0, it_rep = 0;
    const float delta = (float)a.inner_tol;
    while (status == COLAGB_SYS_RUNNING) {
      // A: A p into zq ; <p, A p>
      const float paf = diag_product<CL, G4, float>(cl, ctx, zq, A, a.off, a.nd, ps, true);
      arrived = false;
      float qa[1] = {paf};
      float4 rown[G4];  // r's own rows, loaded while the reduction's barrier completes
      {
        float* sl = next_fslot();
        cluster_sum_f_begin<1, CL>(cl, qa, wpart, sl);
#pragma unroll
        for (int j = 0; j < G4; ++j) rown[j] = ld4(rs + 4 * (tid + j * kOT));
        cluster_sum_f_end<1, CL>(qa, sl);
      }
      const float pap = qa[0];
      if (!(pap > 0.f)) {  // not SPD in FP32 (or NaN)
        status = (pap == pap) ? COLAGB_SYS_BREAKDOWN : COLAGB_SYS_NAN;
        break;
      }
      const float alpha = gamma / pap;
      // B: r -= alpha A p ; |r|^2 ; z and <r, z> (FSAI: after r's halo is published).  All loads of
      // a phase are issued before its first store: the compiler cannot prove that the shared-memory
      // stores do not alias the global loads, and interleaving them would serialise one L2 round
      // trip per row.
      float rrf = 0.f, rzf = 0.f;
#pragma unroll
      for (int h = 0; h < 2; ++h) {  // two halves of the groups: half the registers in flight
        constexpr int H4 = G4 / 2;
        float4 rv[H4], dv[H4];
#pragma unroll
        for (int jj = 0; jj < H4; ++jj) {
          const int j = edge_first<G4>(h * H4 + jj);
          rv[jj] = rown[j];
          dv[jj] = prec == COLAGB_PREC_JACOBI ? ld4(Dv + i0 + 4 * (tid + j * kOT)) : make_float4(1.f, 1.f, 1.f, 1.f);
        }
#pragma unroll
        for (int jj = 0; jj < H4; ++jj) {
          const int j = edge_first<G4>(h * H4 + jj);
          rv[jj].x -= alpha * zq[j].x;
          rv[jj].y -= alpha * zq[j].y;
          rv[jj].z -= alpha * zq[j].z;
          rv[jj].w -= alpha * zq[j].w;
          rrf += dot4(rv[jj], rv[jj]);
          if (prec != COLAGB_PREC_FSAI) {
            const float4 zv = prec == COLAGB_PREC_JACOBI
                                  ? make_float4(dv[jj].x * rv[jj].x, dv[jj].y * rv[jj].y, dv[jj].z * rv[jj].z,
                                                dv[jj].w * rv[jj].w)
                                  : rv[jj];
            zq[j] = zv;
            rzf += dot4(rv[jj], zv);
          }
        }
#pragma unroll
        for (int jj = 0; jj < H4; ++jj) {
          const int j = edge_first<G4>(h * H4 + jj);
          st4(rs + 4 * (tid + j * kOT), rv[jj]);
          if (prec == COLAGB_PREC_FSAI) push_group<CL, G4>(cl, ctx, rs, j);  // M r reads r's halo
        }
      }
      float qb[2] = {rrf, rzf};
      if (prec == COLAGB_PREC_FSAI) {
        push_halos_wide<CL, G4>(cl, ctx, rs);
        __syncthreads();
        cluster_arrive();
        qb[1] = apply_z<CL, G4>(cl, ctx, zq, prec, a, M, Dv, rs, true);
      }
      cluster_sum_f<2, CL>(cl, qb, wpart, next_fslot());
      ++it;
      rn = sqrtf(qb[0]);
      float gamma_new = qb[1];
      bool restart = false, dpend = true;
      if (!(rn == rn)) {
#pragma unroll 1
        for (int l = tid; l < R; l += kOT) ds[l] += alpha * ps[l];
        status = COLAGB_SYS_NAN;
        break;
      }
      if (rn <= delta * rmax || rn <= (float)a.tol || it >= a.max_inner ||
          (a.fallback && prec == COLAGB_PREC_FSAI && it - it_rep >= kJudgeSteps)) {
        // FP64 replacement: x += d + alpha p, d = 0 ; r = b/|b| - A x  (eight rows' x loads in flight)
#pragma unroll 1
        for (int l0 = tid; l0 < R; l0 += kRowBatch * kOT) {
          double xv[kRowBatch];
#pragma unroll
          for (int u = 0; u < kRowBatch; ++u) {
            const int64_t i = i0 + l0 + u * kOT;
            xv[u] = i < n ? X[i] : 0.0;
          }
#pragma unroll
          for (int u = 0; u < kRowBatch; ++u) {
            const int l = l0 + u * kOT;
            const int64_t i = i0 + l;
            const int sl = sidx(l, S);
            const float dn = ds[sl] + alpha * ps[sl];
            if (i < n) X[i] = xv[u] + (double)dn;
            ds[sl] = 0.f;
          }
        }
        dpend = false;
        it_rep = it;
        cl.sync();
        residual(q2[0]);
        cluster_sum<1, CL>(cl, q2, next_slot(), red, bcast);
        ++nrep;
        const double rr = sqrt(q2[0]);
        relres = rr;
        if (!(rr == rr)) { status = COLAGB_SYS_NAN; break; }
        if (rr <= a.tol) { status = COLAGB_SYS_CONVERGED; break; }
        if (it >= a.max_inner || nrep >= a.max_sweeps) { status = COLAGB_SYS_MAX_ITERS; break; }
        if (a.fallback && prec == COLAGB_PREC_FSAI && rr > 0.5 * relres_prev) {
          prec = COLAGB_PREC_JACOBI;  // the FP64 residual judged the learned factor
          restart = true;
        }
        if (a.mode == COLAGB_IR_RESTART) restart = true;
        relres_prev = rr;
        rn = (float)rr;
        rmax = rn;
        if (prec == COLAGB_PREC_FSAI) fill_halo<CL>(cl, ctx, rs);
        __syncthreads();
        q1[0] = apply_z<CL, G4>(cl, ctx, zq, prec, a, M, Dv, rs, false);
        cluster_sum_f<1, CL>(cl, q1, wpart, next_fslot());
        gamma_new = q1[0];
      }
      const float beta = restart || gamma == 0.f ? 0.f : gamma_new / gamma;
      gamma = gamma_new;
      // C: d += alpha p (unless flushed) ; p = z + beta p
#pragma unroll
      for (int h = 0; h < 2; ++h) {  // two halves of the groups: half the registers in flight
        constexpr int H4 = G4 / 2;
        float4 po[H4], dd[H4];
#pragma unroll
        for (int jj = 0; jj < H4; ++jj) {
          const int j = edge_first<G4>(h * H4 + jj);
          po[jj] = ld4(ps + 4 * (tid + j * kOT));
          dd[jj] = ld4(ds + 4 * (tid + j * kOT));
        }
#pragma unroll
        for (int jj = 0; jj < H4; ++jj) {
          const int j = edge_first<G4>(h * H4 + jj);
          st4(ps + 4 * (tid + j * kOT), make_float4(zq[j].x + beta * po[jj].x, zq[j].y + beta * po[jj].y,
                                                    zq[j].z + beta * po[jj].z, zq[j].w + beta * po[jj].w));
          if (dpend)
            st4(ds + 4 * (tid + j * kOT), make_float4(dd[jj].x + alpha * po[jj].x, dd[jj].y + alpha * po[jj].y,
                                                      dd[jj].z + alpha * po[jj].z, dd[jj].w + alpha * po[jj].w));
          push_group<CL, G4>(cl, ctx, ps, j);
        }
      }
      push_halos_wide<CL, G4>(cl, ctx, ps);
      __syncthreads();
      cluster_arrive();  // p and its halos published; waited for at the start of the next step
      arrived = true;
    }
    // every break leaves the loop with no arrive outstanding; a system that needs no step (zero or
    // already-converged right-hand side) still owes the wait for the arrive issued before the loop
    if (arrived) cluster_wait();
    // finish: x += d, scale by |b|
#pragma unroll 1
    for (int l0 = tid; l0 < R; l0 += kRowBatch * kOT) {
      double xv[kRowBatch];
#pragma unroll
      for (int u = 0; u < kRowBatch; ++u) {
        const int64_t i = i0 + l0 + u * kOT;
        xv[u] = i < n ? X[i] : 0.0;
      }
#pragma unroll
      for (int u = 0; u < kRowBatch; ++u) {
        const int l = l0 + u * kOT;
        const int64_t i = i0 + l;
        if (i < n) X[i] = (xv[u] + (double)ds[sidx(l, S)]) * (bnorm > 0.0 ? bnorm : 1.0);
      }
    }
    if (rank == 0 && tid == 0) {
      int st = status == COLAGB_SYS_RUNNING ? COLAGB_SYS_MAX_ITERS : status;
      if (st == COLAGB_SYS_CONVERGED && a.prec_kind == COLAGB_PREC_FSAI && prec != COLAGB_PREC_FSAI)
        st = COLAGB_SYS_FALLBACK;
      if (a.out_status) a.out_status[s] = st;
      if (a.out_iters) a.out_iters[s] = it;
      if (a.out_relres) a.out_relres[s] = relres;
      if (a.out_nrep) a.out_nrep[s] = nrep;
    }
  }
}

// ---------------------------------------------------------------------------------------------
// Companion schedule on the SMs the clusters leave free.  The on-chip clusters hold 16 SMs each
// (7 clusters = 112 of the 152 SMs at 224 KB of shared memory per CTA); on each remaining SM one
// 512-thread CTA solves whole systems alone, with the same algorithm and stop rule, its vectors in
// global memory.  It claims systems from the on-chip kernel's counter while more than `reserve`
// remain unclaimed, so that the clusters (about ten times faster per system) finish the tail.
//
// Layout per CTA: the system's rows padded to np (a multiple of 4 * kST * kRowBatch) in the strip
// layout of the on-chip schedule with the CTA as the whole "cluster" (S = np / 4 float4 groups), so
// every operand of a diagonal product is one aligned 128-bit load; p and r carry a halo of H float4s
// on each side whose components are copies of the adjacent strips' rows, written by the owner of
// each row as it stores it (put4 / put1).  Per step and row the CTA streams the matrix diagonals (A
// in FP32, the FSAI operator M in bfloat16) and ~9 FP32 vector words; the next batches of each
// stream are prefetched into L2 with bulk prefetches so that DRAM latency is hidden without
// registers.  Reductions are block-wide in a fixed order.
constexpr int kST = 512;  // threads per spare-SM CTA
constexpr int kSU = 4;    // float4 groups per thread per batch (loads in flight per stream)
constexpr int64_t kSpareRowAlign = 4 * kST * kRowBatch;  // 16384
constexpr int kSpareRatio = 28;  // cluster solves per companion solve (measured: ~14 ms vs ~380 ms per 512 x 512 system)

struct SpareArgs {
  float* base;       // per-CTA regions of per_cta floats
  int64_t per_cta;
  int64_t np;        // rows padded to kSpareRowAlign
  int H;             // halo float4s on each side (multiple of 4 rows, <= np / 4)
  int reserve;       // claim only while more than this many systems are unclaimed
  unsigned int* solved;  // systems these CTAs solved
};

// floats of one spare CTA's region for n rows: A diagonals, 1/diag, G diagonals, M (bfloat16, in
// float-sized space), p and r with halos of up to np / 4 float4s, A p, z, d.
static int64_t spare_rows(int64_t n) { return (n + kSpareRowAlign - 1) / kSpareRowAlign * kSpareRowAlign; }
static int64_t spare_cta_floats(int64_t n, bool fsai) {
  const int64_t np = spare_rows(n);
  const int64_t mat = (kMaxDiagA + 1) * np + (fsai ? kMaxDiagG * np + (kMaxDiagM * np + 1) / 2 : 0);
  return mat + 2 * (3 * np) + 3 * np + 64;
}

// The companion CTAs' streams carry an L2 evict-first policy: their working sets (~20 MB per system)
// pass through L2 once per step and must not displace the clusters' diagonal slots, which L2 serves
// every ~14 us.
__device__ __forceinline__ uint64_t evict_first_policy() {
  uint64_t pol;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
  return pol;
}
__device__ __forceinline__ void l2_prefetch(const void* p, uint32_t bytes, uint64_t pol) {
  asm volatile("cp.async.bulk.prefetch.L2.global.L2::cache_hint [%0], %1, %2;" ::"l"(p), "r"(bytes), "l"(pol)
               : "memory");
}
__device__ __forceinline__ float4 ld4_ef(const float* p, uint64_t pol) {
  float4 v;
  asm volatile("ld.global.L1::no_allocate.L2::cache_hint.v4.f32 {%0, %1, %2, %3}, [%4], %5;"
               : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
               : "l"(p), "l"(pol));
  return v;
}
__device__ __forceinline__ void st4_ef(float* p, float4 v, uint64_t pol) {
  asm volatile("st.global.L2::cache_hint.v4.f32 [%0], {%1, %2, %3, %4}, %5;" ::"l"(p), "f"(v.x), "f"(v.y), "f"(v.z),
               "f"(v.w), "l"(pol)
               : "memory");
}
template <typename T> struct SpareDiag;
template <> struct SpareDiag<float> {
  using Reg = float4;
  static __device__ __forceinline__ Reg load(const float* p, uint64_t pol) { return ld4_ef(p, pol); }
};
template <> struct SpareDiag<__nv_bfloat16> {
  using Reg = uint2;
  static __device__ __forceinline__ Reg load(const __nv_bfloat16* p, uint64_t pol) {
    uint2 v;
    asm volatile("ld.global.L1::no_allocate.L2::cache_hint.v2.u32 {%0, %1}, [%2], %3;"
                 : "=r"(v.x), "=r"(v.y)
                 : "l"(p), "l"(pol));
    return v;
  }
};

// Strip-layout store of float4 group q of a vector with halos (H float4s each side): the halo
// components that copy q's rows are written too (components 1..3 of the left halo float4 q - S and
// 0..2 of the right halo float4 q + S; the others stay zero from the setup).
__device__ __forceinline__ void put4(float* v, int q, int S, int H, float4 x, uint64_t pol) {
  st4_ef(v + 4 * (int64_t)q, x, pol);
  if (q >= S - H) {
    float* h = v + 4 * (q - S);
    h[1] = x.x;
    h[2] = x.y;
    h[3] = x.z;
  }
  if (q < H) {
    float* h = v + 4 * (q + S);
    h[0] = x.y;
    h[1] = x.z;
    h[2] = x.w;
  }
}
// The same for one row l (float index sidx(l, S)).
__device__ __forceinline__ void put1(float* v, int l, int S, int H, float x) {
  const int q = l % S, c = l / S;
  v[4 * q + c] = x;
  if (q >= S - H && c <= 2) v[4 * (q - S) + c + 1] = x;
  if (q < H && c >= 1) v[4 * (q + S) + c - 1] = x;
}

// Block-wide sums of NQ values in a fixed order (every thread gets the totals).
template <int NQ, class T>
__device__ __forceinline__ void spare_sum(T (&v)[NQ], T* red) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < NQ; ++q) v[q] = warp_sum(v[q]);
  if (lane == 0)
#pragma unroll
    for (int q = 0; q < NQ; ++q) red[q * (kST / 32) + w] = v[q];
  __syncthreads();
#pragma unroll
  for (int q = 0; q < NQ; ++q) {
    T s = T(0);
    for (int u = 0; u < kST / 32; ++u) s += red[q * (kST / 32) + u];
    v[q] = s;
  }
  __syncthreads();
}

// out[q] = sum_k D[k][q] * v[q + off[k]] over this thread's groups (main diagonal last); returns the
// thread's part of <v, D v>.  While a batch is consumed, the batch two ahead of every stream is
// prefetched into L2 (thread k < nk: diagonal k; thread nk: v).
template <typename T>
__device__ __forceinline__ float spare_product(const T* D, const int* off, int nk, int64_t np, const float* v,
                                               float* out, int S, int H, int tid, uint64_t pol) {
  using DL = Diag4<T>;
  using SL = SpareDiag<T>;
  constexpr int kBatch = kSU * kST;  // float4 groups per batch
  float dot = 0.f;
#pragma unroll 1
  for (int g0 = 0; g0 < S; g0 += kBatch) {
    const int gp = g0 + 2 * kBatch;
    if (gp < S) {
      if (tid < nk) l2_prefetch(D + tid * np + 4 * (int64_t)gp, (uint32_t)(kBatch * 4 * sizeof(T)), pol);
      else if (tid == nk) {
        const int lo = gp - H, hi = gp + kBatch + H < S + H ? gp + kBatch + H : S + H;
        l2_prefetch(v + 4 * (int64_t)lo, (uint32_t)((hi - lo) * 16), pol);
      }
    }
    float4 acc[kSU];
#pragma unroll
    for (int u = 0; u < kSU; ++u) acc[u] = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll 1
    for (int k = 0; k < nk; ++k) {
      const T* Dk = D + k * np;
      const int o = off[k];
      typename DL::Reg dv[kSU];
      float4 pv[kSU];
#pragma unroll
      for (int u = 0; u < kSU; ++u) {
        const int q = g0 + tid + u * kST;
        dv[u] = SL::load(Dk + 4 * (int64_t)q, pol);
        pv[u] = ld4_ef(v + 4 * (int64_t)(q + o), pol);
      }
#pragma unroll
      for (int u = 0; u < kSU; ++u) {
        const float4 av = DL::wide(dv[u]);
        acc[u].x = fmaf(av.x, pv[u].x, acc[u].x);
        acc[u].y = fmaf(av.y, pv[u].y, acc[u].y);
        acc[u].z = fmaf(av.z, pv[u].z, acc[u].z);
        acc[u].w = fmaf(av.w, pv[u].w, acc[u].w);
        // the main diagonal comes last: its operand is v's own rows and acc is complete
        if (o == 0 && k == nk - 1) dot += dot4(pv[u], acc[u]);
      }
    }
#pragma unroll
    for (int u = 0; u < kSU; ++u) {
      const int q = g0 + tid + u * kST;
      if (off[nk - 1] != 0) dot += dot4(ld4_ef(v + 4 * (int64_t)q, pol), acc[u]);
      st4_ef(out + 4 * (int64_t)q, acc[u], pol);
    }
  }
  return dot;
}

// Data written inside this kernel by other threads of the CTA is read after a __syncthreads.
__global__ void __launch_bounds__(kST, 1) k_spare_pcg(const __grid_constant__ OnchipArgs a,
                                                      const __grid_constant__ SpareArgs sp) {
  __shared__ double dred[4 * (kST / 32)];
  __shared__ float fred[4 * (kST / 32)];
  __shared__ unsigned int s_sys;
  const int tid = threadIdx.x;
  const int64_t n = a.n, np = sp.np;
  const int S = (int)(np / 4), H = sp.H;
  constexpr int kBatch = kSU * kST;
  float* base = sp.base + (int64_t)blockIdx.x * sp.per_cta;
  float* A = base;
  float* Dv = A + kMaxDiagA * np;
  float* Gd = a.gdia ? Dv + np : nullptr;
  __nv_bfloat16* M = a.mdia ? reinterpret_cast<__nv_bfloat16*>(Dv + np + kMaxDiagG * np) : nullptr;
  float* vec = Dv + np + (a.gdia ? kMaxDiagG * np + (kMaxDiagM * np + 1) / 2 : 0);
  vec = reinterpret_cast<float*>((reinterpret_cast<uintptr_t>(vec) + 15) & ~uintptr_t(15));
  float* ps = vec + 4 * (int64_t)H;             // p: float4 indices [-H, S + H)
  float* rs = ps + 4 * ((int64_t)S + 2 * H);    // r: float4 indices [-H, S + H)
  float* aps = rs + 4 * ((int64_t)S + H);       // A p: [0, S)
  float* zs = aps + np;                         // z (FSAI): [0, S)
  float* ds = zs + np;                          // d: [0, S)
  const uint64_t pol = evict_first_policy();

  while (true) {
    if (tid == 0) {
      unsigned int c = *reinterpret_cast<volatile unsigned int*>(a.next);
      unsigned int got = (unsigned int)a.S;
#pragma unroll 1
      for (int tries = 0; tries < (1 << 20); ++tries) {  // every failed exchange saw a newer claim
        if ((int64_t)c + sp.reserve >= a.S) break;
        const unsigned int prev = atomicCAS(a.next, c, c + 1);
        if (prev == c) {
          got = c;
          break;
        }
        c = prev;
      }
      s_sys = got;
    }
    __syncthreads();
    const int64_t s = s_sys;
    __syncthreads();
    if (s >= a.S) break;

    const float* vals = a.vals + s * a.vstride;
    const double* B = a.B + s * n;
    double* X = a.X + s * n;
    int prec = a.prec_kind;

    // ---- setup: diagonal storage, x = 0, vectors and halos zero, |b|^2 ----
    double v1[1] = {0.0};
#pragma unroll 1
    for (int64_t l = tid; l < np; l += kST) {
      const bool live = l < n;
      const int64_t si = sidx((int)l, S);
      csr_row_to_diagonals(a.indptr, a.indices, vals, l, live, a.off, a.nd, A + si, np);
      Dv[si] = a.center >= 0 && A[a.center * np + si] != 0.f ? 1.f / A[a.center * np + si] : 1.f;
      if (Gd) csr_row_to_diagonals(a.g_indptr, a.g_indices, a.g_vals + s * a.g_nnz, l, live, a.goff, a.ng, Gd + l, np);
      ps[l] = 0.f;
      rs[l] = 0.f;
      ds[l] = 0.f;
      if (l < 4 * H) {
        ps[l - 4 * H] = 0.f;
        ps[np + l] = 0.f;
        rs[l - 4 * H] = 0.f;
        rs[np + l] = 0.f;
      }
      if (live) {
        const double bv = B[l];
        v1[0] += bv * bv;
        X[l] = 0.0;
      }
    }
    spare_sum<1>(v1, dred);  // also publishes G's diagonals and x = 0 to the CTA
    if (M) {  // M = G^T G (same construction as the clusters', CTA = whole system)
#pragma unroll 1
      for (int l0 = tid; l0 < np; l0 += kRowBatch * kST) {
        float asum[kRowBatch], ctr[kRowBatch];
#pragma unroll
        for (int u = 0; u < kRowBatch; ++u) asum[u] = ctr[u] = 0.f;
        int mc = 0;
#pragma unroll 1
        for (int m = 0; m < a.nm; ++m) {
          float v[kRowBatch];
#pragma unroll
          for (int u = 0; u < kRowBatch; ++u) v[u] = 0.f;
#pragma unroll 1
          for (int q = a.pstart[m]; q < a.pstart[m + 1]; ++q) {
            const float* ga = Gd + a.pa[q] * np;
            const float* gb = Gd + a.pb[q] * np;
            const int go = a.goff[a.pa[q]];
#pragma unroll
            for (int u = 0; u < kRowBatch; ++u) {
              const int64_t i = l0 + u * kST;
              const int64_t k = i - go;
              if (i < n && k < n) v[u] += ga[k] * gb[k];
            }
          }
#pragma unroll
          for (int u = 0; u < kRowBatch; ++u) asum[u] += fabsf(v[u]);
          if (a.moff[m] == 0) {
            mc = m;
#pragma unroll
            for (int u = 0; u < kRowBatch; ++u) ctr[u] = v[u];
          } else {
#pragma unroll
            for (int u = 0; u < kRowBatch; ++u) M[m * np + sidx(l0 + u * kST, S)] = __float2bfloat16_rn(v[u]);
          }
        }
#pragma unroll
        for (int u = 0; u < kRowBatch; ++u)
          M[mc * np + sidx(l0 + u * kST, S)] = __float2bfloat16_rn(ctr[u] + kMBoost * asum[u]);
      }
    }
    const double bnorm = sqrt(v1[0]);
    int status = COLAGB_SYS_RUNNING;
    double relres = bnorm > 0.0 ? 1.0 : 0.0;
    if (!(bnorm > 0.0)) status = bnorm == 0.0 ? COLAGB_SYS_CONVERGED : COLAGB_SYS_NAN;
    const double binv = bnorm > 0.0 ? 1.0 / bnorm : 1.0;

    // r = b/|b| - A x in FP64 (eight rows' loads in flight per diagonal), |r|^2; r's halos too
    auto residual = [&](double& rr) {
      rr = 0.0;
#pragma unroll 1
      for (int l0 = tid; l0 < np; l0 += kRowBatch * kST) {
        double ax[kRowBatch];
#pragma unroll
        for (int u = 0; u < kRowBatch; ++u) ax[u] = 0.0;
#pragma unroll 1
        for (int k = 0; k < a.nd; ++k) {
          const float* Ak = A + k * np;
          const int o = a.off[k];
#pragma unroll
          for (int u = 0; u < kRowBatch; ++u) {
            const int l = l0 + u * kST;
            const int64_t c = (int64_t)l + o;
            const float av = Ak[sidx(l, S)];
            const double xv = c >= 0 && c < n ? X[c] : 0.0;
            ax[u] += (double)av * xv;
          }
        }
#pragma unroll
        for (int u = 0; u < kRowBatch; ++u) {
          const int l = l0 + u * kST;
          if (l < n) {
            const double rv = B[l] * binv - ax[u];
            put1(rs, l, S, H, (float)rv);
            rr += rv * rv;
          }
        }
      }
    };
    // z (preconditioned r) into dst with its halos when dst is p, into zs (FSAI) otherwise; <r, z>
    auto precondition = [&](float* dst) -> float {
      float rz = 0.f;
      if (prec == COLAGB_PREC_FSAI) {
        rz = spare_product<__nv_bfloat16>(M, a.moff, a.nm, np, rs, zs, S, H, tid, pol);
        if (dst == ps) {
          __syncthreads();
#pragma unroll 1
          for (int q = tid; q < S; q += kST) put4(ps, q, S, H, ld4_ef(zs + 4 * (int64_t)q, pol), pol);
        }
        return rz;
      }
#pragma unroll 1
      for (int q = tid; q < S; q += kST) {
        const float4 r = ld4_ef(rs + 4 * (int64_t)q, pol);
        float4 z = r;
        if (prec == COLAGB_PREC_JACOBI) {
          const float4 d = ld4_ef(Dv + 4 * (int64_t)q, pol);
          z = make_float4(d.x * r.x, d.y * r.y, d.z * r.z, d.w * r.w);
        }
        rz += dot4(r, z);
        if (dst == ps) put4(ps, q, S, H, z, pol);
      }
      return rz;
    };

    double q2[1];
    residual(q2[0]);
    spare_sum<1>(q2, dred);  // r and its halos complete
    float rn = (float)sqrt(q2[0]);
    float rmax = rn;
    double relres_prev = relres;
    float q1[1] = {precondition(ps)};
    spare_sum<1>(q1, fred);  // p and its halos complete
    float gamma = q1[0];
    if (status == COLAGB_SYS_RUNNING && rn <= (float)a.tol) status = COLAGB_SYS_CONVERGED;

    int it = 0, nrep = 0, it_rep = 0;
    const float delta = (float)a.inner_tol;
    while (status == COLAGB_SYS_RUNNING) {
      // A: A p ; <p, A p>
      float qa[1] = {spare_product<float>(A, a.off, a.nd, np, ps, aps, S, H, tid, pol)};
      spare_sum<1>(qa, fred);
      const float pap = qa[0];
      if (!(pap > 0.f)) {
        status = (pap == pap) ? COLAGB_SYS_BREAKDOWN : COLAGB_SYS_NAN;
        break;
      }
      const float alpha = gamma / pap;
      // B: r -= alpha A p ; |r|^2 ; <r, z> (Jacobi / none here, FSAI after r is complete)
      float rrf = 0.f, rzf = 0.f;
#pragma unroll 1
      for (int g0 = 0; g0 < S; g0 += kBatch) {
        float4 rv[kSU], av[kSU], dv[kSU];
#pragma unroll
        for (int u = 0; u < kSU; ++u) {
          const int64_t q = g0 + tid + u * kST;
          rv[u] = ld4_ef(rs + 4 * q, pol);
          av[u] = ld4_ef(aps + 4 * q, pol);
          dv[u] = prec == COLAGB_PREC_JACOBI ? ld4_ef(Dv + 4 * q, pol) : make_float4(1.f, 1.f, 1.f, 1.f);
        }
#pragma unroll
        for (int u = 0; u < kSU; ++u) {
          const int q = g0 + tid + u * kST;
          rv[u].x -= alpha * av[u].x;
          rv[u].y -= alpha * av[u].y;
          rv[u].z -= alpha * av[u].z;
          rv[u].w -= alpha * av[u].w;
          rrf += dot4(rv[u], rv[u]);
          if (prec != COLAGB_PREC_FSAI) {
            const float4 zv = prec == COLAGB_PREC_JACOBI
                                  ? make_float4(dv[u].x * rv[u].x, dv[u].y * rv[u].y, dv[u].z * rv[u].z,
                                                dv[u].w * rv[u].w)
                                  : rv[u];
            rzf += dot4(rv[u], zv);
          }
          put4(rs, q, S, H, rv[u], pol);
        }
      }
      float qb[2] = {rrf, rzf};
      if (prec == COLAGB_PREC_FSAI) {
        __syncthreads();  // r and its halos complete
        qb[1] = precondition(zs);
      }
      spare_sum<2>(qb, fred);
      ++it;
      rn = sqrtf(qb[0]);
      float gamma_new = qb[1];
      bool restart = false, dpend = true;
      if (!(rn == rn)) {
#pragma unroll 1
        for (int64_t l = tid; l < np; l += kST) ds[l] += alpha * ps[l];
        status = COLAGB_SYS_NAN;
        break;
      }
      if (rn <= delta * rmax || rn <= (float)a.tol || it >= a.max_inner ||
          (a.fallback && prec == COLAGB_PREC_FSAI && it - it_rep >= kJudgeSteps)) {
        // FP64 replacement: x += d + alpha p, d = 0 ; r = b/|b| - A x
#pragma unroll 1
        for (int l0 = tid; l0 < np; l0 += kRowBatch * kST) {
          double xv[kRowBatch];
#pragma unroll
          for (int u = 0; u < kRowBatch; ++u) {
            const int64_t i = l0 + u * kST;
            xv[u] = i < n ? X[i] : 0.0;
          }
#pragma unroll
          for (int u = 0; u < kRowBatch; ++u) {
            const int l = l0 + u * kST;
            const int sl = sidx(l, S);
            const float dn = ds[sl] + alpha * ps[sl];
            if (l < n) X[l] = xv[u] + (double)dn;
            ds[sl] = 0.f;
          }
        }
        dpend = false;
        it_rep = it;
        __syncthreads();  // x complete before any thread reads its neighbours' rows
        residual(q2[0]);
        spare_sum<1>(q2, dred);
        ++nrep;
        const double rr = sqrt(q2[0]);
        relres = rr;
        if (!(rr == rr)) { status = COLAGB_SYS_NAN; break; }
        if (rr <= a.tol) { status = COLAGB_SYS_CONVERGED; break; }
        if (it >= a.max_inner || nrep >= a.max_sweeps) { status = COLAGB_SYS_MAX_ITERS; break; }
        if (a.fallback && prec == COLAGB_PREC_FSAI && rr > 0.5 * relres_prev) {
          prec = COLAGB_PREC_JACOBI;
          restart = true;
        }
        if (a.mode == COLAGB_IR_RESTART) restart = true;
        relres_prev = rr;
        rn = (float)rr;
        rmax = rn;
        q1[0] = precondition(zs);
        spare_sum<1>(q1, fred);
        gamma_new = q1[0];
      }
      const float beta = restart || gamma == 0.f ? 0.f : gamma_new / gamma;
      gamma = gamma_new;
      // C: d += alpha p (unless flushed) ; p = z + beta p, with p's halos
#pragma unroll 1
      for (int g0 = 0; g0 < S; g0 += kBatch) {
        float4 po[kSU], dd[kSU], zv[kSU];
#pragma unroll
        for (int u = 0; u < kSU; ++u) {
          const int64_t q = g0 + tid + u * kST;
          po[u] = ld4_ef(ps + 4 * q, pol);
          dd[u] = ld4_ef(ds + 4 * q, pol);
          if (prec == COLAGB_PREC_FSAI) {
            zv[u] = ld4_ef(zs + 4 * q, pol);
          } else {
            const float4 r = ld4_ef(rs + 4 * q, pol);
            if (prec == COLAGB_PREC_JACOBI) {
              const float4 d = ld4_ef(Dv + 4 * q, pol);
              zv[u] = make_float4(d.x * r.x, d.y * r.y, d.z * r.z, d.w * r.w);
            } else {
              zv[u] = r;
            }
          }
        }
#pragma unroll
        for (int u = 0; u < kSU; ++u) {
          const int q = g0 + tid + u * kST;
          if (dpend)
            st4_ef(ds + 4 * (int64_t)q, make_float4(dd[u].x + alpha * po[u].x, dd[u].y + alpha * po[u].y,
                                                    dd[u].z + alpha * po[u].z, dd[u].w + alpha * po[u].w), pol);
          put4(ps, q, S, H, make_float4(zv[u].x + beta * po[u].x, zv[u].y + beta * po[u].y,
                                        zv[u].z + beta * po[u].z, zv[u].w + beta * po[u].w), pol);
        }
      }
      __syncthreads();  // p and its halos complete
    }
    __syncthreads();
    // finish: x += d, scale by |b|
#pragma unroll 1
    for (int l0 = tid; l0 < np; l0 += kRowBatch * kST) {
      double xv[kRowBatch];
#pragma unroll
      for (int u = 0; u < kRowBatch; ++u) {
        const int64_t i = l0 + u * kST;
        xv[u] = i < n ? X[i] : 0.0;
      }
#pragma unroll
      for (int u = 0; u < kRowBatch; ++u) {
        const int l = l0 + u * kST;
        if (l < n) X[l] = (xv[u] + (double)ds[sidx(l, S)]) * (bnorm > 0.0 ? bnorm : 1.0);
      }
    }
    if (tid == 0) {
      int st = status == COLAGB_SYS_RUNNING ? COLAGB_SYS_MAX_ITERS : status;
      if (st == COLAGB_SYS_CONVERGED && a.prec_kind == COLAGB_PREC_FSAI && prec != COLAGB_PREC_FSAI)
        st = COLAGB_SYS_FALLBACK;
      if (a.out_status) a.out_status[s] = st;
      if (a.out_iters) a.out_iters[s] = it;
      if (a.out_relres) a.out_relres[s] = relres;
      if (a.out_nrep) a.out_nrep[s] = nrep;
      atomicAdd(sp.solved, 1u);
    }
    __syncthreads();
  }
}

// ---- pattern analysis: the set of diagonals (column - row) a CSR pattern occupies ----
__global__ void k_offset_bitmap(const int32_t* __restrict__ indptr, const int32_t* __restrict__ indices, int64_t n,
                                unsigned int* bits) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    for (int32_t e = indptr[i]; e < indptr[i + 1]; ++e) {
      const int64_t o = (int64_t)indices[e] - i + (n - 1);  // [0, 2n - 2] for valid columns
      if (o >= 0 && o < 2 * n - 1) atomicOr(bits + (o >> 5), 1u << (o & 31));
    }
}

// out[0] = number of distinct diagonals, out[1 .. 32] = the first 32 offsets in ascending order.
__global__ void k_offset_collect(const unsigned int* __restrict__ bits, int64_t nwords, int64_t n, int* out) {
  __shared__ int cnt[1024];
  const int t = threadIdx.x;
  const int64_t per = (nwords + blockDim.x - 1) / blockDim.x;
  const int64_t w0 = t * per, w1 = (w0 + per < nwords) ? w0 + per : nwords;
  int c = 0;
  for (int64_t w = w0; w < w1; ++w) c += __popc(bits[w]);
  cnt[t] = c;
  __syncthreads();
  if (t == 0) {
    int acc = 0;
    for (int u = 0; u < (int)blockDim.x; ++u) {
      const int v = cnt[u];
      cnt[u] = acc;
      acc += v;
    }
    out[0] = acc;
  }
  __syncthreads();
  int rnk = cnt[t];
  for (int64_t w = w0; w < w1 && rnk < 32; ++w) {
    unsigned int b = bits[w];
    while (b && rnk < 32) {
      const int bit = __ffs(b) - 1;
      b &= b - 1;
      out[1 + rnk] = (int)(w * 32 + bit - (n - 1));
      ++rnk;
    }
  }
}

static int diag_offsets(const int32_t* indptr, const int32_t* indices, int64_t n, unsigned int* bits, int* dout,
                        std::vector<int>& offs, cudaStream_t st) {
  const int64_t nwords = (2 * n - 1 + 31) / 32;
  COLAGB_CUDA(cudaMemsetAsync(bits, 0, nwords * sizeof(unsigned int), st));
  const int nb = (int)std::min<int64_t>((n + 255) / 256, 4 * (int64_t)num_sms());
  k_offset_bitmap<<<nb, 256, 0, st>>>(indptr, indices, n, bits);
  COLAGB_CUDA(cudaGetLastError());
  k_offset_collect<<<1, 1024, 0, st>>>(bits, nwords, n, dout);
  COLAGB_CUDA(cudaGetLastError());
  int h[33];
  COLAGB_CUDA(cudaMemcpyAsync(h, dout, sizeof(h), cudaMemcpyDeviceToHost, st));
  COLAGB_CUDA(cudaStreamSynchronize(st));
  offs.assign(h + 1, h + 1 + std::min(h[0], 32));
  if (h[0] > 32) offs.push_back(0);  // more than 32: marks the pattern as not diagonal-structured
  return COLAGB_OK;
}

// Dynamic shared memory per CTA: p and r with their halos (S + 2H float4s each, S = R / 4), d.
static size_t onchip_smem_bytes(int R, int H) { return (size_t)(3 * R + 16 * H) * sizeof(float); }

// Cluster size and rows per CTA for the on-chip schedule, from n alone (also used to size the
// workspace).  Returns 0 when n is too large to keep p, r and d on chip.
static int onchip_cluster(int64_t n, int* rows_per_cta, int* groups) {
  for (int cl : {8, 16}) {
    const int64_t r = (n + cl - 1) / cl;
    for (int g : {8, 16, 32}) {
      if (r <= (int64_t)kOT * g) {
        if (rows_per_cta) *rows_per_cta = kOT * g;
        if (groups) *groups = g;
        if ((size_t)3 * kOT * g * sizeof(float) <= kOnchipSmemMax) return cl;
      }
    }
  }
  return 0;
}

static int onchip_slots(int cl) { return (num_sms() + cl - 1) / cl; }

template <int CL, int G>
static int onchip_active_clusters(size_t smem, int* nclusters);

// CTAs of the companion schedule: the SMs that the clusters leave free at the largest shared-memory
// footprint (the fewest resident clusters), 0 when none.
static int spare_ctas(int64_t n) {
  int R = 0, G = 0;
  const int CL = onchip_cluster(n, &R, &G);
  if (CL == 0) return 0;
  int nc = 0;
  if (CL == 8)
    G == 8 ? onchip_active_clusters<8, 8>(kOnchipSmemMax, &nc)
           : G == 16 ? onchip_active_clusters<8, 16>(kOnchipSmemMax, &nc) : onchip_active_clusters<8, 32>(kOnchipSmemMax, &nc);
  else
    G == 8 ? onchip_active_clusters<16, 8>(kOnchipSmemMax, &nc)
           : G == 16 ? onchip_active_clusters<16, 16>(kOnchipSmemMax, &nc) : onchip_active_clusters<16, 32>(kOnchipSmemMax, &nc);
  if (nc < 1) return 0;
  const int free_sms = num_sms() - CL * std::min(nc, onchip_slots(CL));
  return free_sms > 0 ? free_sms : 0;
}

// Workspace of the on-chip schedule (diagonal slots + pattern scratch, then the companion CTAs'
// regions); 0 when not applicable.
size_t onchip_workspace_floats(int64_t n, bool fsai, bool spare) {
  int R = 0;
  const int cl = onchip_cluster(n, &R, nullptr);
  if (cl == 0) return 0;
  const int64_t np = (int64_t)cl * R;
  const int64_t per = kMaxDiagA + 1 + (fsai ? kMaxDiagG + kMaxDiagM : 0);
  const size_t core = (size_t)onchip_slots(cl) * per * np + (size_t)(2 * n + 31) / 32 + 64 + 64;
  return spare ? core + 64 + (size_t)spare_ctas(n) * spare_cta_floats(n, fsai) : core;
}

// A private non-blocking stream and two events per CUDA context for the companion launch (forked
// from and joined back into the caller's stream).
struct SpareStreams {
  unsigned long long ctx = 0;
  cudaStream_t st = nullptr;
  cudaEvent_t fork = nullptr, join = nullptr;
};
static const SpareStreams* spare_streams() {
  static std::mutex mu;
  static std::vector<SpareStreams> all;
  const unsigned long long id = current_context_id();
  if (id == 0) return nullptr;
  std::lock_guard<std::mutex> lk(mu);
  for (const auto& e : all)
    if (e.ctx == id) return &e;
  SpareStreams e;
  e.ctx = id;
  // load the companion kernel now: with lazy module loading its first launch would otherwise load it
  // then, which waits for the clusters' kernel already running, and the companions would start late
  cudaFuncAttributes fa;
  if (cudaFuncGetAttributes(&fa, k_spare_pcg) != cudaSuccess ||
      cudaStreamCreateWithFlags(&e.st, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&e.fork, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&e.join, cudaEventDisableTiming) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  all.reserve(64);
  if (all.size() >= 64) return nullptr;  // keeps the returned pointers stable
  all.push_back(e);
  return &all.back();
}

template <int CL, int G>
static int launch_onchip(const OnchipArgs& a, size_t smem, cudaStream_t st) {
  auto kern = k_onchip_pcg<CL, G>;
  COLAGB_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  if (CL > 8) COLAGB_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = CL;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cfg.blockDim = dim3(kOT);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cfg.gridDim = dim3((unsigned)(CL * onchip_slots(CL)));
  int nclusters = 0;
  if (cudaOccupancyMaxActiveClusters(&nclusters, kern, &cfg) != cudaSuccess || nclusters < 1) {
    cudaGetLastError();
    return fail(COLAGB_ERR_UNSUPPORTED, "on-chip PCG: cluster not schedulable");
  }
  int64_t nc = std::min<int64_t>(std::min<int64_t>(nclusters, onchip_slots(CL)), a.S);
  cfg.gridDim = dim3((unsigned)(CL * nc));
  COLAGB_CUDA(cudaLaunchKernelEx(&cfg, kern, a));
  return COLAGB_OK;
}

template <int CL, int G>
static int onchip_active_clusters(size_t smem, int* nclusters) {
  auto kern = k_onchip_pcg<CL, G>;
  COLAGB_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  if (CL > 8) COLAGB_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = CL;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cfg.blockDim = dim3(kOT);
  cfg.dynamicSmemBytes = smem;
  cfg.gridDim = dim3((unsigned)(CL * onchip_slots(CL)));
  *nclusters = 0;
  if (cudaOccupancyMaxActiveClusters(nclusters, kern, &cfg) != cudaSuccess) {
    cudaGetLastError();
    *nclusters = 0;
  }
  return COLAGB_OK;
}

// Called by colagb_cg_batched_csr_solve.  Returns COLAGB_ERR_UNSUPPORTED (without launching) when
// the pattern is not a handful of diagonals or the system does not fit on chip; `*used` tells the
// caller whether it ran.
int onchip_pcg_solve(const colagb_batched_csr* Acsr, const double* B, double* X, const colagb_ir_params* prm,
                     int32_t* iters, int32_t* status, double* relres, int* nrep, void* ws, size_t ws_bytes,
                     bool* used, unsigned int** companion_solved, cudaStream_t st) {
  *used = false;
  *companion_solved = nullptr;
  const int64_t n = Acsr->n;
  const bool fsai = prm->preconditioner == COLAGB_PREC_FSAI;
  int R = 0, G = 0;
  const int CL = onchip_cluster(n, &R, &G);
  if (CL == 0 || n < 1) return COLAGB_OK;
  const bool want_spare = prm->spare != COLAGB_SPARE_OFF;
  const size_t need = onchip_workspace_floats(n, fsai, want_spare) * sizeof(float);
  if (ws_bytes < need || ws == nullptr) return COLAGB_OK;
  const int nspare = want_spare ? spare_ctas(n) : 0;
  const int64_t np = (int64_t)CL * R;
  const int64_t per = kMaxDiagA + 1 + (fsai ? kMaxDiagG + kMaxDiagM : 0);
  float* base = static_cast<float*>(ws);
  const size_t slots = (size_t)onchip_slots(CL);
  float* adia = base;
  float* gdia = fsai ? adia + slots * kMaxDiagA * np : nullptr;
  float* mdia = fsai ? gdia + slots * kMaxDiagG * np : nullptr;
  float* dinv = adia + slots * (kMaxDiagA + (fsai ? kMaxDiagG + kMaxDiagM : 0)) * np;
  unsigned int* bits = reinterpret_cast<unsigned int*>(base + slots * per * np);
  int* dout = reinterpret_cast<int*>(bits + (2 * n + 31) / 32);
  unsigned int* counter = reinterpret_cast<unsigned int*>(dout + 64);

  std::vector<int> off, goff;
  COLAGB_TRY(diag_offsets(Acsr->indptr, Acsr->indices, n, bits, dout, off, st));
  if (off.empty() || (int)off.size() > kMaxDiagA) return COLAGB_OK;
  // the main diagonal last: its operand is then the thread's own rows, still in registers when the
  // product is complete, for <v, D v> (diag_product)
  std::stable_partition(off.begin(), off.end(), [](int o) { return o != 0; });
  OnchipArgs a = {};
  a.nd = (int)off.size();
  a.center = -1;
  int H = 0;
  for (int k = 0; k < a.nd; ++k) {
    a.off[k] = off[k];
    if (off[k] == 0) a.center = k;
    H = std::max(H, std::abs(off[k]));
  }
  if (fsai) {
    COLAGB_TRY(diag_offsets(Acsr->g_indptr, Acsr->g_indices, n, bits, dout, goff, st));
    if (goff.empty() || (int)goff.size() > kMaxDiagG) return COLAGB_OK;
    for (int o : goff)
      if (o > 0) return COLAGB_OK;  // G must be lower triangular
    std::vector<int> moff;
    for (int o1 : goff)
      for (int o2 : goff) moff.push_back(o2 - o1);
    std::sort(moff.begin(), moff.end());
    moff.erase(std::unique(moff.begin(), moff.end()), moff.end());
    if ((int)moff.size() > kMaxDiagM) return COLAGB_OK;
    std::stable_partition(moff.begin(), moff.end(), [](int o) { return o != 0; });  // main diagonal last
    a.ng = (int)goff.size();
    a.nm = (int)moff.size();
    for (int k = 0; k < a.ng; ++k) a.goff[k] = goff[k];
    int q = 0;
    for (int m = 0; m < a.nm; ++m) {
      a.moff[m] = moff[m];
      H = std::max(H, std::abs(moff[m]));
      a.pstart[m] = q;
      for (int i1 = 0; i1 < a.ng; ++i1)
        for (int i2 = 0; i2 < a.ng; ++i2)
          if (goff[i2] - goff[i1] == moff[m]) {
            if (q >= kMaxPairs) return COLAGB_OK;
            a.pa[q] = i1;
            a.pb[q] = i2;
            ++q;
          }
    }
    a.pstart[a.nm] = q;
  }
  H = (H + 3) / 4 * 4;  // halo rows in whole 16-byte words
  if (H > R / 4) return COLAGB_OK;  // a halo reaches at most one strip (strip layout)
  const size_t smem = onchip_smem_bytes(R, H);
  if (smem > kOnchipSmemMax) return COLAGB_OK;

  a.n = n;
  a.S = Acsr->num_systems;
  a.np = np;
  a.R = R;
  a.H = H;
  a.indptr = Acsr->indptr;
  a.indices = Acsr->indices;
  a.vals = Acsr->values;
  a.vstride = Acsr->shared_values ? 0 : Acsr->nnz;
  a.g_indptr = Acsr->g_indptr;
  a.g_indices = Acsr->g_indices;
  a.g_vals = Acsr->g_values;
  a.g_nnz = Acsr->g_nnz;
  a.adia = adia;
  a.gdia = gdia;
  a.mdia = mdia;
  a.dinv = dinv;
  a.next = counter;
  a.B = B;
  a.X = X;
  a.out_status = status;
  a.out_iters = iters;
  a.out_relres = relres;
  a.out_nrep = nrep;
  a.tol = prm->tol;
  a.inner_tol = prm->inner_tol;
  a.max_sweeps = prm->max_sweeps;
  a.max_inner = prm->max_inner_iters;
  a.prec_kind = prm->preconditioner;
  a.fallback = prm->fallback;
  a.mode = prm->mode;
  COLAGB_CUDA(cudaMemsetAsync(counter, 0, 2 * sizeof(unsigned int), st));  // system counter, companion count
  *companion_solved = counter + 1;
  // companion CTAs on the free SMs (prm->spare: AUTO, OFF, or ONLY for tests)
  const int spare_mode = prm->spare;
  const int64_t nps = spare_rows(n);
  const SpareStreams* ss = nullptr;
  int nsp = 0;
  if (spare_mode != COLAGB_SPARE_OFF && nspare > 0 && H <= nps / 4) {
    ss = spare_streams();
    if (ss) nsp = nspare;
  }
  if (spare_mode == COLAGB_SPARE_ONLY && nsp == 0) return COLAGB_OK;  // not available: the caller falls back
  SpareArgs sp = {};
  if (nsp > 0) {
    sp.base = reinterpret_cast<float*>((reinterpret_cast<uintptr_t>(counter + 16) + 255) & ~uintptr_t(255));
    sp.per_cta = spare_cta_floats(n, fsai);
    sp.np = nps;
    sp.H = H;
    sp.solved = counter + 1;
    // a cluster solves a system ~kSpareRatio times faster than one CTA does: leave the clusters that many
    // systems each at the end, so that no companion solve outlasts the clusters' last one
    int nc = 0;
    if (CL == 8)
      G == 8 ? onchip_active_clusters<8, 8>(smem, &nc)
             : G == 16 ? onchip_active_clusters<8, 16>(smem, &nc) : onchip_active_clusters<8, 32>(smem, &nc);
    else
      G == 8 ? onchip_active_clusters<16, 8>(smem, &nc)
             : G == 16 ? onchip_active_clusters<16, 16>(smem, &nc) : onchip_active_clusters<16, 32>(smem, &nc);
    nsp = std::min<int64_t>(std::max(0, num_sms() - CL * std::min(nc, onchip_slots(CL))), nspare);
    sp.reserve = spare_mode == COLAGB_SPARE_ONLY ? 0 : (int)std::min<int64_t>((int64_t)kSpareRatio * nc, 1 << 30);
    if (spare_mode != COLAGB_SPARE_ONLY && (nsp == 0 || a.S <= sp.reserve)) nsp = 0;
    if (spare_mode == COLAGB_SPARE_ONLY && nsp == 0) nsp = nspare;
  }
  if (nsp > 0) COLAGB_CUDA(cudaEventRecord(ss->fork, st));
  int rc = COLAGB_OK;
  if (spare_mode == COLAGB_SPARE_ONLY) {
    // no clusters: the companion CTAs take every system
  } else if (CL == 8)
    rc = G == 8 ? launch_onchip<8, 8>(a, smem, st)
                : G == 16 ? launch_onchip<8, 16>(a, smem, st) : launch_onchip<8, 32>(a, smem, st);
  else
    rc = G == 8 ? launch_onchip<16, 8>(a, smem, st)
                : G == 16 ? launch_onchip<16, 16>(a, smem, st) : launch_onchip<16, 32>(a, smem, st);
  if (rc == COLAGB_OK && nsp > 0) {
    COLAGB_CUDA(cudaStreamWaitEvent(ss->st, ss->fork, 0));
    k_spare_pcg<<<(unsigned)nsp, kST, 0, ss->st>>>(a, sp);
    COLAGB_CUDA(cudaGetLastError());
    COLAGB_CUDA(cudaEventRecord(ss->join, ss->st));
    COLAGB_CUDA(cudaStreamWaitEvent(st, ss->join, 0));
  }
  if (rc == COLAGB_OK) *used = true;
  return rc == COLAGB_ERR_UNSUPPORTED ? COLAGB_OK : rc;
}

}  // namespace colagb

using namespace colagb;

extern "C" int colagb_onchip_schedule_info(int64_t n, int32_t halo, int32_t* info) {
  if (!info || n < 0 || halo < 0) return fail(COLAGB_ERR_INVALID, "onchip info: bad argument");
  int R = 0, G = 0;
  const int CL = onchip_cluster(n, &R, &G);
  info[0] = CL;
  info[1] = R;
  info[2] = 0;
  info[3] = 0;
  if (CL == 0) return COLAGB_OK;
  const int H = (halo + 3) / 4 * 4;
  const size_t smem = onchip_smem_bytes(R, H);
  info[3] = (int32_t)smem;
  if (smem > kOnchipSmemMax || H > R / 4) return COLAGB_OK;
  int nc = 0, rc;
  if (CL == 8)
    rc = G == 8 ? onchip_active_clusters<8, 8>(smem, &nc)
                : G == 16 ? onchip_active_clusters<8, 16>(smem, &nc) : onchip_active_clusters<8, 32>(smem, &nc);
  else
    rc = G == 8 ? onchip_active_clusters<16, 8>(smem, &nc)
                : G == 16 ? onchip_active_clusters<16, 16>(smem, &nc) : onchip_active_clusters<16, 32>(smem, &nc);
  COLAGB_TRY(rc);
  info[2] = std::min(nc, onchip_slots(CL));
  return COLAGB_OK;
}
