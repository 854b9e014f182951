// Batched independent SPD systems sharing one CSR sparsity pattern, solved to a true FP64 relative
// residual by FP32 preconditioned CG with FP64 iterative refinement -- one persistent launch.
//
// Per system s the inner loop is the reference's PCG step (cola/linalg/inverse/cg.py:141-170,
// with P = Diagonal(1/diag A) for Jacobi or P = G^T G for FSAI); the reference solves each system
// with its own cola.linalg.solve(PSD(Sparse), b, CG(P=...)) call (inv.py:24-69).
//
// Precision scheme (per system, b normalised to |b| = 1):
//   FP32 vectors r, p, Ap, d, z; FP64 solution x.
//   Every CG step: d += alpha p, r -= alpha Ap (FP32).
//   Replacement, when |r| has dropped by inner_tol since the last one, or |r| <= tol:
//       x += d, d = 0 (FP64);  r = b - A x  (FP64 arithmetic on the FP32 stored values);
//       relres = |b - A x| (FP64) -- the only convergence test (relres <= tol).
//   COLAGB_IR_RELIABLE: the CG recurrence continues with the replaced residual (reliable updates,
//   no Krylov restart).  COLAGB_IR_RESTART: every replacement also restarts CG (p = z), the classic
//   refinement sweep.
// The FP64 true residual also judges the learned preconditioner: a system whose FSAI segment fails
// to halve its true residual continues with Jacobi (status COLAGB_SYS_FALLBACK).
//
// Work distribution: every phase splits the active systems into q row chunks each (~8 chunks per
// CTA) and gives each CTA a contiguous range of chunks, so a CTA mostly stays inside one system and
// reduces its per-system sums once; rows are processed 4 per thread per step with all loads issued
// before any store (memory-level parallelism for the HBM-bound streams).
#include <string>
#include <vector>

#include "common.cuh"

namespace colagb {

constexpr int kMaxBatch = 1024;  // systems per launch (host splits larger batches)
constexpr int kThreads = 256;
constexpr int kUnroll = 4;
constexpr int kRowUnroll = 6;    // CSR entries per row handled without a loop

struct BatchedArgs {
  int64_t n, nnz, S;
  int64_t vstride;  // elements between systems' value arrays (0: one shared matrix)
  const int32_t* __restrict__ indptr;
  const int32_t* __restrict__ indices;
  const float* __restrict__ vals;
  int64_t g_nnz;
  const int32_t* g_indptr;
  const int32_t* g_indices;
  const int32_t* gt_indptr;
  const int32_t* gt_indices;
  const int32_t* gt_perm;
  const float* g_vals;
  const double* B;
  double* X;                             // FP64 solution (in units of |b| until the final scaling)
  float *r, *p, *ap, *d, *z, *t, *dinv;  // [S][n]
  double* acc;                           // [6][S]
  double* bnorm;                         // [S]
  int* out_status;
  int* out_iters;
  double* out_relres;
  int* summary;  // [0] max replacements, [1] max iterations
  double tol, inner_tol;
  int max_sweeps, max_inner, prec_kind, fallback, mode;
  GridBarrier gb;
};

// per-system state, identical in every CTA: one shared-memory block addressed from a single base
// pointer (FP64 fields first, then 32-bit fields), S entries per field
struct SysState {
  unsigned char* base;
  int S;
  __device__ __forceinline__ double* f64(int k) const { return reinterpret_cast<double*>(base) + (size_t)k * S; }
  __device__ __forceinline__ float* f32(int k) const {
    return reinterpret_cast<float*>(base + (size_t)3 * 8 * S) + (size_t)k * S;
  }
  __device__ __forceinline__ int* i32(int k) const {
    return reinterpret_cast<int*>(base + (size_t)3 * 8 * S) + (size_t)(4 + k) * S;
  }
  __device__ __forceinline__ double& gamma(int s) const { return f64(0)[s]; }
  __device__ __forceinline__ double& relres(int s) const { return f64(1)[s]; }
  __device__ __forceinline__ double& relres_prev(int s) const { return f64(2)[s]; }
  __device__ __forceinline__ float& alpha(int s) const { return f32(0)[s]; }
  __device__ __forceinline__ float& beta(int s) const { return f32(1)[s]; }
  __device__ __forceinline__ float& rn(int s) const { return f32(2)[s]; }
  __device__ __forceinline__ float& rmax(int s) const { return f32(3)[s]; }
  __device__ __forceinline__ int& status(int s) const { return i32(0)[s]; }
  __device__ __forceinline__ int& prec(int s) const { return i32(1)[s]; }
  __device__ __forceinline__ int& it(int s) const { return i32(2)[s]; }
  __device__ __forceinline__ int& nrep(int s) const { return i32(3)[s]; }
  __device__ __forceinline__ int& flags(int s) const { return i32(4)[s]; }
  __device__ __forceinline__ int* act() const { return i32(5); }
  __device__ __forceinline__ int* act2() const { return i32(6); }
  __device__ __forceinline__ int& it_rep(int s) const { return i32(7)[s]; }
};
constexpr int F_ACTIVE = 1, F_REPLACE = 2, F_RESTART = 4;

__device__ __forceinline__ void chunking(int nact, int nb, int64_t n, int& q, int64_t& cs) {
  const int target = 8 * nb;
  q = nact > 0 ? (target + nact - 1) / nact : 1;
  if (q < 1) q = 1;
  if ((int64_t)q > n) q = (int)n;
  cs = (n + q - 1) / q;
  cs = (cs + 3) / 4 * 4;  // row chunks start on 16-byte boundaries (vector phases)
  q = (int)((n + cs - 1) / cs);
}

// the per-system FP64 accumulators: acc[k][s] = base[k * S + s]
struct AccSet {
  double* base;
  int S;
  __device__ __forceinline__ double* operator[](int k) const { return base + (size_t)k * S; }
  __device__ __forceinline__ AccSet operator+(int k) const { return AccSet{base + (size_t)k * S, S}; }
};

template <class A, int NA>
__device__ __forceinline__ void flush(int s, A* v, const AccSet& acc, A* red) {
#pragma unroll
  for (int k = 0; k < NA; ++k) {
    const A x = block_sum(v[k], red);
    if (threadIdx.x == 0) atomicAdd(acc[k] + s, (double)x);
    v[k] = A(0);
  }
}

// Runs functor f over every (system, row) of the active list.  f.load(s, i) issues the loads of one
// row, f.finish(s, i, l, v) computes, stores and adds NA contributions to v.  Per-system sums go to
// acc[k][s] (FP64 atomics, once per CTA and system).
template <class A, int NA, class F>
__device__ __forceinline__ void sweep(const int* act, int nact, int64_t n, const F& f, const AccSet& acc, A* red) {
  if (nact <= 0) return;
  int q;
  int64_t cs;
  chunking(nact, gridDim.x, n, q, cs);
  const int64_t total = (int64_t)nact * q;
  const int64_t c0 = total * blockIdx.x / gridDim.x, c1 = total * (blockIdx.x + 1) / gridDim.x;
  int cur = -1;
  A v[NA > 0 ? NA : 1];
#pragma unroll
  for (int k = 0; k < (NA > 0 ? NA : 1); ++k) v[k] = A(0);
  for (int64_t ch = c0; ch < c1; ++ch) {
    const int s = act[ch / q];
    if (NA > 0 && s != cur) {
      if (cur >= 0) flush<A, NA>(cur, v, acc, red);
      cur = s;
    }
    const int64_t i0 = (ch % q) * cs;
    const int64_t i1 = (i0 + cs < n) ? i0 + cs : n;
    constexpr int U = F::kU;
    if constexpr (F::kVec == 4) {
      // 4 consecutive rows per thread with 128-bit loads (n % 4 == 0 is checked by the host)
      for (int64_t base = i0 + 4 * (int64_t)threadIdx.x; base < i1; base += 4 * (int64_t)kThreads) {
        const typename F::L l = f.load(s, base);
        f.finish(s, base, l, v);
      }
    } else {
      for (int64_t base = i0 + threadIdx.x; base < i1; base += U * kThreads) {
        typename F::L l[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const int64_t i = base + (int64_t)u * kThreads;
          if (i < i1) l[u] = f.load(s, i);
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const int64_t i = base + (int64_t)u * kThreads;
          if (i < i1) f.finish(s, i, l[u], v);
        }
      }
    }
  }
  if (NA > 0 && cur >= 0) flush<A, NA>(cur, v, acc, red);
}

// CSR row dot with up to kRowUnroll entries unrolled (predicated), the rest in a loop.  `x` is
// rewritten by other CTAs during the kernel, so it must not be declared __restrict__ (that would let
// the compiler read it through the non-coherent read-only cache and see stale values).
template <class T, class V>
__device__ __forceinline__ T csr_dot(const int32_t* __restrict__ indptr, const int32_t* __restrict__ indices,
                                     const float* __restrict__ vals, const V* x, int64_t i) {
  const int32_t b = __ldg(indptr + i), e = __ldg(indptr + i + 1);
  T acc = T(0);
#pragma unroll
  for (int k = 0; k < kRowUnroll; ++k) {
    const int32_t j = b + k;
    if (j < e) acc += (T)vals[j] * (T)x[__ldg(indices + j)];
  }
  for (int32_t j = b + kRowUnroll; j < e; ++j) acc += (T)vals[j] * (T)x[__ldg(indices + j)];
  return acc;
}

__device__ __forceinline__ float apply_m_row(const BatchedArgs& a, int pk, int64_t s, int64_t i, float rv) {
  if (pk == COLAGB_PREC_JACOBI) return a.dinv[s * a.n + i] * rv;
  return rv;
}

// ---- phase functors -----------------------------------------------------------------------------
struct FMatvec {
  static constexpr int kVec = 1;
  static constexpr int kU = 2;  // Ap = A p ; <p, Ap>
  const BatchedArgs* a;
  struct L { float pv, ap; };
  __device__ __forceinline__ L load(int s, int64_t i) const {
    const int64_t so = (int64_t)s * a->n;
    L l;
    l.ap = csr_dot<float, float>(a->indptr, a->indices, a->vals + (int64_t)s * a->vstride, a->p + so, i);
    l.pv = a->p[so + i];
    return l;
  }
  __device__ __forceinline__ void finish(int s, int64_t i, const L& l, float* v) const {
    a->ap[(int64_t)s * a->n + i] = l.ap;
    v[0] += l.pv * l.ap;
  }
};

struct FUpdate {  // d += alpha p ; r -= alpha Ap ; |r|^2 ; <r, M r> for Jacobi / none   (4 rows)
  static constexpr int kVec = 4;
  static constexpr int kU = 1;
  const BatchedArgs* a;
  const SysState* m;
  struct L { float4 d, p, r, ap, di; };
  __device__ __forceinline__ L load(int s, int64_t i) const {
    const int64_t u = (int64_t)s * a->n + i;
    L l;
    l.d = *reinterpret_cast<const float4*>(a->d + u);
    l.p = *reinterpret_cast<const float4*>(a->p + u);
    l.r = *reinterpret_cast<const float4*>(a->r + u);
    l.ap = *reinterpret_cast<const float4*>(a->ap + u);
    l.di = (m->prec(s) == COLAGB_PREC_JACOBI) ? *reinterpret_cast<const float4*>(a->dinv + u)
                                              : make_float4(1.f, 1.f, 1.f, 1.f);
    return l;
  }
  __device__ __forceinline__ void finish(int s, int64_t i, const L& l, float* v) const {
    const int64_t u = (int64_t)s * a->n + i;
    const float al = m->alpha(s);
    float4 d, r;
    d.x = l.d.x + al * l.p.x; d.y = l.d.y + al * l.p.y; d.z = l.d.z + al * l.p.z; d.w = l.d.w + al * l.p.w;
    r.x = l.r.x - al * l.ap.x; r.y = l.r.y - al * l.ap.y; r.z = l.r.z - al * l.ap.z; r.w = l.r.w - al * l.ap.w;
    *reinterpret_cast<float4*>(a->d + u) = d;
    *reinterpret_cast<float4*>(a->r + u) = r;
    v[0] += r.x * r.x + r.y * r.y + r.z * r.z + r.w * r.w;
    v[1] += r.x * (l.di.x * r.x) + r.y * (l.di.y * r.y) + r.z * (l.di.z * r.z) + r.w * (l.di.w * r.w);
  }
};

struct FFlushX {  // x += d ; d = 0   (4 rows)
  static constexpr int kVec = 4;
  static constexpr int kU = 1;
  const BatchedArgs* a;
  struct L { double2 x0, x1; float4 d; };
  __device__ __forceinline__ L load(int s, int64_t i) const {
    const int64_t u = (int64_t)s * a->n + i;
    L l;
    l.x0 = *reinterpret_cast<const double2*>(a->X + u);
    l.x1 = *reinterpret_cast<const double2*>(a->X + u + 2);
    l.d = *reinterpret_cast<const float4*>(a->d + u);
    return l;
  }
  __device__ __forceinline__ void finish(int s, int64_t i, const L& l, double*) const {
    const int64_t u = (int64_t)s * a->n + i;
    *reinterpret_cast<double2*>(a->X + u) = make_double2(l.x0.x + (double)l.d.x, l.x0.y + (double)l.d.y);
    *reinterpret_cast<double2*>(a->X + u + 2) = make_double2(l.x1.x + (double)l.d.z, l.x1.y + (double)l.d.w);
    *reinterpret_cast<float4*>(a->d + u) = make_float4(0.f, 0.f, 0.f, 0.f);
  }
};

struct FResidual {
  static constexpr int kVec = 1;
  static constexpr int kU = 1;  // r = b/|b| - A x in FP64 ; |r|^2 (FP64) ; <r, M r> for Jacobi / none
  const BatchedArgs* a;
  const SysState* m;
  struct L { double ax, b; float di; };
  __device__ __forceinline__ L load(int s, int64_t i) const {
    const int64_t so = (int64_t)s * a->n;
    L l;
    l.ax = csr_dot<double, double>(a->indptr, a->indices, a->vals + (int64_t)s * a->vstride, a->X + so, i);
    l.b = a->B[so + i];
    l.di = (m->prec(s) == COLAGB_PREC_JACOBI) ? a->dinv[so + i] : 1.f;
    return l;
  }
  __device__ __forceinline__ void finish(int s, int64_t i, const L& l, double* v) const {
    const double rv = l.b / a->bnorm[s] - l.ax;
    const float rf = (float)rv;
    a->r[(int64_t)s * a->n + i] = rf;
    v[0] += rv * rv;
    v[1] += (double)(rf * (l.di * rf));
  }
};

struct FFsaiT {
  static constexpr int kVec = 1;
  static constexpr int kU = 2;  // t = G r (FSAI systems)
  const BatchedArgs* a;
  const SysState* m;
  struct L { float t; };
  __device__ __forceinline__ L load(int s, int64_t i) const {
    L l{0.f};
    if (m->prec(s) != COLAGB_PREC_FSAI) return l;
    const float* g = a->g_vals + (int64_t)s * a->g_nnz;
    const float* rs = a->r + (int64_t)s * a->n;
    for (int32_t e = a->g_indptr[i]; e < a->g_indptr[i + 1]; ++e) l.t += g[e] * rs[a->g_indices[e]];
    return l;
  }
  __device__ __forceinline__ void finish(int s, int64_t i, const L& l, float*) const {
    if (m->prec(s) == COLAGB_PREC_FSAI) a->t[(int64_t)s * a->n + i] = l.t;
  }
};

struct FZ {
  static constexpr int kVec = 1;
  static constexpr int kU = 2;  // z = M r (G^T t for FSAI) ; <r, z>
  const BatchedArgs* a;
  const SysState* m;
  struct L { float z, r; };
  __device__ __forceinline__ L load(int s, int64_t i) const {
    const int64_t u = (int64_t)s * a->n + i;
    L l;
    l.r = a->r[u];
    const int pk = m->prec(s);
    if (pk == COLAGB_PREC_FSAI) {
      const float* g = a->g_vals + (int64_t)s * a->g_nnz;
      const float* ts = a->t + (int64_t)s * a->n;
      float v = 0.f;
      for (int32_t e = a->gt_indptr[i]; e < a->gt_indptr[i + 1]; ++e) v += g[a->gt_perm[e]] * ts[a->gt_indices[e]];
      l.z = v;
    } else {
      l.z = apply_m_row(*a, pk, s, i, l.r);
    }
    return l;
  }
  __device__ __forceinline__ void finish(int s, int64_t i, const L& l, float* v) const {
    a->z[(int64_t)s * a->n + i] = l.z;
    v[0] += l.r * l.z;
  }
};

struct FPUpdate {  // p = z + beta p  (z stored, or M r recomputed)   (4 rows)
  static constexpr int kVec = 4;
  static constexpr int kU = 1;
  const BatchedArgs* a;
  const SysState* m;
  bool zstored;
  struct L { float4 z, p; };
  __device__ __forceinline__ L load(int s, int64_t i) const {
    const int64_t u = (int64_t)s * a->n + i;
    L l;
    if (zstored) {
      l.z = *reinterpret_cast<const float4*>(a->z + u);
    } else {
      l.z = *reinterpret_cast<const float4*>(a->r + u);
      if (m->prec(s) == COLAGB_PREC_JACOBI) {
        const float4 di = *reinterpret_cast<const float4*>(a->dinv + u);
        l.z.x *= di.x; l.z.y *= di.y; l.z.z *= di.z; l.z.w *= di.w;
      }
    }
    l.p = *reinterpret_cast<const float4*>(a->p + u);
    return l;
  }
  __device__ __forceinline__ void finish(int s, int64_t i, const L& l, float*) const {
    const float b = m->beta(s);
    // beta = 0 (first direction, restarts): p = z without touching the old p, which is
    // uninitialised workspace before the first step (0 * NaN would be NaN)
    *reinterpret_cast<float4*>(a->p + (int64_t)s * a->n + i) =
        b == 0.f ? l.z : make_float4(l.z.x + b * l.p.x, l.z.y + b * l.p.y, l.z.z + b * l.p.z, l.z.w + b * l.p.w);
  }
};

struct FSetup {
  static constexpr int kVec = 1;
  static constexpr int kU = 1;  // |b|^2 ; x = 0 ; d = 0 ; Jacobi diagonal
  const BatchedArgs* a;
  struct L { double b; float dg; };
  __device__ __forceinline__ L load(int s, int64_t i) const {
    const int64_t u = (int64_t)s * a->n + i;
    L l;
    l.b = a->B[u];
    l.dg = 0.f;
    if (a->dinv) {
      const float* vals = a->vals + (int64_t)s * a->vstride;
      for (int32_t j = a->indptr[i]; j < a->indptr[i + 1]; ++j)
        if (a->indices[j] == i) l.dg += vals[j];
    }
    return l;
  }
  __device__ __forceinline__ void finish(int s, int64_t i, const L& l, double* v) const {
    const int64_t u = (int64_t)s * a->n + i;
    if (a->dinv) a->dinv[u] = l.dg != 0.f ? 1.f / l.dg : 1.f;
    a->X[u] = 0.0;
    a->d[u] = 0.f;
    v[0] += l.b * l.b;
  }
};

struct FScaleX {  // X = |b| x   (4 rows)
  static constexpr int kVec = 4;
  static constexpr int kU = 1;
  const BatchedArgs* a;
  struct L { double2 x0, x1; };
  __device__ __forceinline__ L load(int s, int64_t i) const {
    const int64_t u = (int64_t)s * a->n + i;
    return L{*reinterpret_cast<const double2*>(a->X + u), *reinterpret_cast<const double2*>(a->X + u + 2)};
  }
  __device__ __forceinline__ void finish(int s, int64_t i, const L& l, double*) const {
    const int64_t u = (int64_t)s * a->n + i;
    const double b = a->bnorm[s];
    *reinterpret_cast<double2*>(a->X + u) = make_double2(l.x0.x * b, l.x0.y * b);
    *reinterpret_cast<double2*>(a->X + u + 2) = make_double2(l.x1.x * b, l.x1.y * b);
  }
};

template <class P>
__device__ __forceinline__ int build_list(int S, int* list, P pred) {
  __shared__ int s_n;
  __syncthreads();
  if (threadIdx.x == 0) {
    int c = 0;
    for (int s = 0; s < S; ++s)
      if (pred(s)) list[c++] = s;
    s_n = c;
  }
  __syncthreads();
  const int r = s_n;
  __syncthreads();
  return r;
}

__global__ void __launch_bounds__(kThreads, 4) k_batched_ir(const __grid_constant__ BatchedArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int S = (int)a.S;
  const int64_t n = a.n;
  SysState m{smem_raw, S};
  __shared__ float redf[32];
  __shared__ double redd[32];
  AccSet acc{a.acc, S};
  const float delta = (float)a.inner_tol;
  const bool restart_mode = a.mode == COLAGB_IR_RESTART;

  auto zero_acc = [&](int k) {
    if (blockIdx.x == 0)
      for (int s = threadIdx.x; s < S; s += blockDim.x) acc[k][s] = 0.0;
  };

  // ---------------- setup ----------------
  for (int s = threadIdx.x; s < S; s += blockDim.x) {
    m.prec(s) = a.prec_kind;
    m.status(s) = COLAGB_SYS_RUNNING;
    m.it(s) = 0;
    m.nrep(s) = 0;
    m.it_rep(s) = 0;
    m.flags(s) = F_ACTIVE;
  }
  int nact = build_list(S, m.act(), [&](int) { return true; });
  sweep<double, 1>(m.act(), nact, n, FSetup{&a}, acc, redd);
  if (!grid_sync(a.gb)) return;
  for (int s = threadIdx.x; s < S; s += blockDim.x) {
    const double bn = sqrt(__ldcg(acc[0] + s));
    if (blockIdx.x == 0) a.bnorm[s] = bn > 0.0 ? bn : 1.0;
    m.relres(s) = bn > 0.0 ? 1.0 : 0.0;
    m.relres_prev(s) = m.relres(s);
    if (!(bn > 0.0)) {
      m.status(s) = (bn == 0.0) ? COLAGB_SYS_CONVERGED : COLAGB_SYS_NAN;
      m.flags(s) = 0;
    }
  }
  __syncthreads();
  if (!grid_sync(a.gb)) return;  // acc[0] read everywhere, bnorm visible
  zero_acc(0);
  nact = build_list(S, m.act(), [&](int s) { return (m.flags(s) & F_ACTIVE) != 0; });
  // r = b/|b| (x = 0): the residual phase with x = 0 computes exactly that, in FP64
  sweep<double, 2>(m.act(), nact, n, FResidual{&a, &m}, acc + 3, redd);
  if (!grid_sync(a.gb)) return;
  bool any_fsai = false;
  for (int j = 0; j < nact; ++j) any_fsai |= m.prec(m.act()[j]) == COLAGB_PREC_FSAI;
  if (any_fsai) {
    sweep<float, 0>(m.act(), nact, n, FFsaiT{&a, &m}, acc, redf);
    if (!grid_sync(a.gb)) return;
  }
  sweep<float, 1>(m.act(), nact, n, FZ{&a, &m}, acc + 5, redf);  // z, <r, z>
  if (!grid_sync(a.gb)) return;
  for (int j = threadIdx.x; j < nact; j += blockDim.x) {
    const int s = m.act()[j];
    m.gamma(s) = __ldcg(acc[5] + s);
    const float rn = (float)sqrt(__ldcg(acc[3] + s));
    m.rn(s) = rn;
    m.rmax(s) = rn;
    m.beta(s) = 0.f;
    if (rn <= (float)a.tol) { m.status(s) = COLAGB_SYS_CONVERGED; m.flags(s) = 0; }
  }
  __syncthreads();
  nact = build_list(S, m.act(), [&](int s) { return (m.flags(s) & F_ACTIVE) != 0; });
  sweep<float, 0>(m.act(), nact, n, FPUpdate{&a, &m, true}, acc, redf);  // p = z
  if (!grid_sync(a.gb)) return;
  zero_acc(3);
  zero_acc(4);
  zero_acc(5);
  if (!grid_sync(a.gb)) return;

  // ---------------- CG iterations ----------------
  int max_rep = 0, max_it = 0;
  while (nact > 0) {
    // Every read of accumulators 1-5 happened before the barrier that closed the previous
    // iteration, and the next writes to them follow at least one more barrier.
    zero_acc(1);
    zero_acc(2);
    zero_acc(3);
    zero_acc(4);
    zero_acc(5);
    // A: Ap = A p, <p, Ap>
    sweep<float, 1>(m.act(), nact, n, FMatvec{&a}, acc, redf);
    if (!grid_sync(a.gb)) return;
    for (int j = threadIdx.x; j < nact; j += blockDim.x) {
      const int s = m.act()[j];
      const double pap = __ldcg(acc[0] + s);
      m.alpha(s) = pap > 0.0 ? (float)(m.gamma(s) / pap) : 0.f;
      if (!(pap > 0.0)) {  // not SPD in FP32 (or NaN): stop this system, keep its last x
        m.status(s) = (pap == pap) ? COLAGB_SYS_BREAKDOWN : COLAGB_SYS_NAN;
        m.flags(s) = 0;
      }
    }
    __syncthreads();
    nact = build_list(S, m.act(), [&](int s) { return (m.flags(s) & F_ACTIVE) != 0; });
    // B: d, r updates, |r|^2, <r, M r>
    sweep<float, 2>(m.act(), nact, n, FUpdate{&a, &m}, acc + 1, redf);
    if (!grid_sync(a.gb)) return;
    zero_acc(0);
    int nrepl = 0;
    if (threadIdx.x == 0) {
      for (int j = 0; j < nact; ++j) {
        const int s = m.act()[j];
        const float rn = (float)sqrt(__ldcg(acc[1] + s));  // FUpdate: acc[1] = |r|^2, acc[2] = <r, M r>
        m.rn(s) = rn;
        m.it(s) += 1;
        int f = m.flags(s) & ~(F_REPLACE | F_RESTART);
        if (!(rn == rn)) {
          m.status(s) = COLAGB_SYS_NAN;
          f = 0;
        } else if (rn <= delta * m.rmax(s) || rn <= (float)a.tol || m.it(s) >= a.max_inner ||
                   (a.fallback && m.prec(s) == COLAGB_PREC_FSAI && m.it(s) - m.it_rep(s) >= kJudgeSteps)) {
          f |= F_REPLACE;
        }
        m.flags(s) = f;
      }
    }
    __syncthreads();
    nrepl = build_list(S, m.act2(), [&](int s) { return (m.flags(s) & F_REPLACE) != 0; });
    if (nrepl > 0) {
      // R1: x += d, d = 0 ; R2: r = b/|b| - A x in FP64
      sweep<double, 0>(m.act2(), nrepl, n, FFlushX{&a}, acc, redd);
      if (!grid_sync(a.gb)) return;
      sweep<double, 2>(m.act2(), nrepl, n, FResidual{&a, &m}, acc + 3, redd);
      if (!grid_sync(a.gb)) return;
      if (threadIdx.x == 0) {
        for (int j = 0; j < nrepl; ++j) {
          const int s = m.act2()[j];
          const double rr = sqrt(__ldcg(acc[3] + s));
          m.nrep(s) += 1;
          m.it_rep(s) = m.it(s);
          int f = m.flags(s);
          if (!(rr == rr)) {
            m.status(s) = COLAGB_SYS_NAN;
            f = 0;
          } else if (rr <= a.tol) {
            m.status(s) = COLAGB_SYS_CONVERGED;
            f = 0;
          } else if (m.it(s) >= a.max_inner || m.nrep(s) >= a.max_sweeps) {
            m.status(s) = COLAGB_SYS_MAX_ITERS;
            f = 0;
          } else {
            if (a.fallback && m.prec(s) == COLAGB_PREC_FSAI && rr > 0.5 * m.relres_prev(s)) {
              m.prec(s) = COLAGB_PREC_JACOBI;  // the FP64 residual judged the learned preconditioner
              f |= F_RESTART;
            }
            if (restart_mode) f |= F_RESTART;
          }
          m.relres_prev(s) = rr;
          m.relres(s) = rr;
          m.rn(s) = (float)rr;
          m.rmax(s) = (float)rr;
          m.flags(s) = f;
        }
      }
      __syncthreads();
    }
    nact = build_list(S, m.act(), [&](int s) { return (m.flags(s) & F_ACTIVE) != 0; });
    if (nact == 0) break;
    any_fsai = false;
    bool switched = false;
    for (int j = 0; j < nact; ++j) {
      const int s = m.act()[j];
      any_fsai |= m.prec(s) == COLAGB_PREC_FSAI;
      switched |= (m.flags(s) & F_RESTART) && a.prec_kind == COLAGB_PREC_FSAI;
    }
    const bool zphase = any_fsai || switched;
    if (any_fsai) {
      sweep<float, 0>(m.act(), nact, n, FFsaiT{&a, &m}, acc, redf);
      if (!grid_sync(a.gb)) return;
    }
    if (zphase) {
      sweep<float, 1>(m.act(), nact, n, FZ{&a, &m}, acc + 5, redf);
      if (!grid_sync(a.gb)) return;
    }
    for (int j = threadIdx.x; j < nact; j += blockDim.x) {
      const int s = m.act()[j];
      const double g1 = zphase ? __ldcg(acc[5] + s)
                               : ((m.flags(s) & F_REPLACE) ? __ldcg(acc[4] + s) : __ldcg(acc[2] + s));
      m.beta(s) = (m.flags(s) & F_RESTART) || m.gamma(s) == 0.0 ? 0.f : (float)(g1 / m.gamma(s));
      m.gamma(s) = g1;
    }
    __syncthreads();
    // C: p = z + beta p
    sweep<float, 0>(m.act(), nact, n, FPUpdate{&a, &m, zphase}, acc, redf);
    if (!grid_sync(a.gb)) return;
  }
  // ---------------- finish: flush d, scale x, report ----------------
  nact = build_list(S, m.act(), [&](int) { return true; });
  sweep<double, 0>(m.act(), nact, n, FFlushX{&a}, acc, redd);
  if (!grid_sync(a.gb)) return;
  sweep<double, 0>(m.act(), nact, n, FScaleX{&a}, acc, redd);
  if (blockIdx.x == 0) {
    for (int s = threadIdx.x; s < S; s += blockDim.x) {
      int st = m.status(s);
      if (st == COLAGB_SYS_RUNNING) st = COLAGB_SYS_MAX_ITERS;
      if (st == COLAGB_SYS_CONVERGED && a.prec_kind == COLAGB_PREC_FSAI && m.prec(s) != COLAGB_PREC_FSAI)
        st = COLAGB_SYS_FALLBACK;
      if (a.out_status) a.out_status[s] = st;
      if (a.out_iters) a.out_iters[s] = m.it(s);
      if (a.out_relres) a.out_relres[s] = m.relres(s);
    }
    if (threadIdx.x == 0) {
      for (int s = 0; s < S; ++s) {
        max_rep = m.nrep(s) > max_rep ? m.nrep(s) : max_rep;
        max_it = m.it(s) > max_it ? m.it(s) : max_it;
      }
      a.summary[0] = max_rep;
      a.summary[1] = max_it;
    }
  }
}

static size_t batched_smem(int64_t S) { return (size_t)S * (3 * 8 + 12 * 4) + 64; }

struct BatchedWs {
  float *r, *p, *ap, *d, *z, *t, *dinv;
  double *acc, *bnorm;
  unsigned int* bar;
  int* summary;
  int* nrep;
  float* onchip;
  size_t onchip_bytes;
  __nv_bfloat16* v16;  // BF16 inner matvec: off-diagonal values and the consistent diagonal
  float* dg16;
  char* block;         // block schedule buffers (cg_block.cu)
  size_t block_bytes;
};

size_t onchip_workspace_floats(int64_t n, bool fsai, bool spare);
size_t block_workspace_bytes(int64_t n, int64_t S, int nb_max);
int block_grid_blocks();
int block_pcg_solve(const colagb_batched_csr* A, const double* B, double* X, const colagb_ir_params* prm,
                    int32_t* iters, int32_t* status, double* relres, void* ws_ptr, size_t ws_bytes, int* max_rep,
                    cudaStream_t st);

// Whether the lockstep block schedule runs: asked for, or AUTO on a shared-values family of >= 4
// right-hand sides with a Jacobi / no preconditioner and the FP32 matvec.
static bool use_block(const colagb_batched_csr& A, const colagb_ir_params& prm) {
  if (prm.schedule == COLAGB_SCHED_BLOCK) return true;
  return prm.schedule == COLAGB_SCHED_AUTO && A.shared_values && A.num_systems >= 4 &&
         prm.preconditioner != COLAGB_PREC_FSAI && prm.matvec == COLAGB_MATVEC_FP32;
}
int onchip_pcg_solve(const colagb_batched_csr* A, const double* B, double* X, const colagb_ir_params* prm,
                     int32_t* iters, int32_t* status, double* relres, int* nrep, void* ws, size_t ws_bytes,
                     bool* used, unsigned int** companion_solved, cudaStream_t st);

static BatchedWs carve_batched(Bump& ws, const colagb_batched_csr& A, const colagb_ir_params& prm) {
  const int64_t S = A.num_systems < kMaxBatch ? A.num_systems : kMaxBatch;
  const int64_t sn = S * A.n;
  BatchedWs w;
  w.r = ws.take<float>(sn);
  w.p = ws.take<float>(sn);
  w.ap = ws.take<float>(sn);
  w.d = ws.take<float>(sn);
  w.z = ws.take<float>(sn);
  const bool fsai = prm.preconditioner == COLAGB_PREC_FSAI;
  const bool jac = prm.preconditioner == COLAGB_PREC_JACOBI || (fsai && prm.fallback);
  w.t = fsai ? ws.take<float>(sn) : nullptr;
  w.dinv = jac ? ws.take<float>(sn) : nullptr;
  w.acc = ws.take<double>(6 * S);
  w.bnorm = ws.take<double>(S);
  w.bar = ws.take<unsigned int>(8);
  w.summary = ws.take<int>(8);
  w.nrep = ws.take<int>(S);
  const bool bf = prm.matvec == COLAGB_MATVEC_BF16;
  if (use_block(A, prm)) {  // the block schedule carves its own buffers
    w.onchip = nullptr;
    w.onchip_bytes = 0;
    w.v16 = nullptr;
    w.dg16 = nullptr;
    const size_t bb = block_workspace_bytes(A.n, A.num_systems, num_sms() * 4);
    w.block = ws.take<char>(bb);
    w.block_bytes = bb;
    return w;
  }
  w.block = nullptr;
  w.block_bytes = 0;
  const bool onchip = !bf && (prm.schedule == COLAGB_SCHED_AUTO || prm.schedule == COLAGB_SCHED_ONCHIP);
  const size_t nf = onchip ? onchip_workspace_floats(A.n, fsai, prm.spare != COLAGB_SPARE_OFF) : 0;
  w.onchip = nf ? ws.take<float>(nf) : nullptr;
  w.onchip_bytes = nf * sizeof(float);
  const int64_t sets = A.shared_values ? 1 : S;
  w.v16 = bf ? ws.take<__nv_bfloat16>((size_t)(sets * A.nnz)) : nullptr;
  w.dg16 = bf ? ws.take<float>((size_t)(sets * A.n)) : nullptr;
  return w;
}

int cluster_pcg_solve(const colagb_batched_csr* A, const double* B, double* X, const colagb_ir_params* prm,
                      int32_t* iters, int32_t* status, double* relres, float* r, float* p, float* ap, float* d,
                      float* z, float* t, float* dinv, int* nrep, int cluster_size, __nv_bfloat16* v16,
                      float* dg16, cudaStream_t st);

// Cluster size for the cluster schedule: 0 = use the cooperative grid kernel.
static int pick_cluster(const colagb_ir_params& prm, int64_t n) {
  if (prm.matvec == COLAGB_MATVEC_BF16 && (prm.schedule == COLAGB_SCHED_AUTO || prm.schedule == COLAGB_SCHED_ONCHIP))
    return n >= 16 * 1024 ? 16 : 8;  // the BF16 inner matvec runs on the cluster schedule
  if (prm.schedule == COLAGB_SCHED_GRID || prm.schedule == COLAGB_SCHED_ONCHIP) return 0;
  if (prm.schedule == COLAGB_SCHED_CLUSTER8) return 8;
  if (prm.schedule == COLAGB_SCHED_CLUSTER16) return 16;
  return n >= 16 * 1024 ? 16 : 8;  // auto: wide clusters for large systems
}

static int validate_batched(const colagb_batched_csr* A, const colagb_ir_params* prm) {
  if (!A || !prm) return fail(COLAGB_ERR_INVALID, "batched CG: null argument");
  if (A->n < 0 || A->nnz < 0 || A->num_systems < 0) return fail(COLAGB_ERR_INVALID, "batched CG: negative size");
  if (A->n > 0 && (!A->indptr || (A->nnz > 0 && (!A->indices || !A->values))))
    return fail(COLAGB_ERR_INVALID, "batched CG: missing CSR arrays");
  if (prm->preconditioner < 0 || prm->preconditioner > 2)
    return fail(COLAGB_ERR_INVALID, "batched CG: unknown preconditioner");
  if (prm->schedule < COLAGB_SCHED_AUTO || prm->schedule > COLAGB_SCHED_BLOCK)
    return fail(COLAGB_ERR_INVALID, "batched CG: unknown schedule");
  if (prm->schedule == COLAGB_SCHED_BLOCK &&
      (!A->shared_values || prm->preconditioner == COLAGB_PREC_FSAI || prm->matvec != COLAGB_MATVEC_FP32))
    return fail(COLAGB_ERR_UNSUPPORTED,
                "batched CG: the block schedule needs a shared-values family, no FSAI and the FP32 matvec");
  if (prm->mode != COLAGB_IR_RELIABLE && prm->mode != COLAGB_IR_RESTART)
    return fail(COLAGB_ERR_INVALID, "batched CG: unknown refinement mode");
  if (prm->preconditioner == COLAGB_PREC_FSAI &&
      (!A->g_indptr || !A->g_indices || !A->gt_indptr || !A->gt_indices || !A->gt_perm || !A->g_values))
    return fail(COLAGB_ERR_INVALID, "batched CG: FSAI preconditioner needs G and G^T patterns and values");
  if (!(prm->tol > 0) || !(prm->inner_tol > 0) || !(prm->inner_tol < 1))
    return fail(COLAGB_ERR_INVALID, "batched CG: need tol > 0 and 0 < inner_tol < 1");
  if (prm->max_sweeps < 0 || prm->max_inner_iters < 0) return fail(COLAGB_ERR_INVALID, "batched CG: negative limits");
  if (prm->matvec != COLAGB_MATVEC_FP32 && prm->matvec != COLAGB_MATVEC_BF16)
    return fail(COLAGB_ERR_INVALID, "batched CG: unknown matvec storage");
  if (prm->matvec == COLAGB_MATVEC_BF16 && (prm->schedule == COLAGB_SCHED_GRID || prm->schedule == COLAGB_SCHED_ONCHIP))
    return fail(COLAGB_ERR_UNSUPPORTED, "batched CG: the BF16 inner matvec runs on the cluster schedules only");
  if (A->n >= (int64_t)1 << 31 || A->nnz >= (int64_t)1 << 31)
    return fail(COLAGB_ERR_INVALID, "batched CG: n and nnz must fit int32 indices");
  return COLAGB_OK;
}

}  // namespace colagb

using namespace colagb;

extern "C" int colagb_cg_batched_csr_workspace_bytes(const colagb_batched_csr* A, const colagb_ir_params* params,
                                                     size_t* bytes) {
  COLAGB_TRY(validate_batched(A, params));
  if (!bytes) return fail(COLAGB_ERR_INVALID, "null bytes");
  Bump ws = Bump::measuring();
  carve_batched(ws, *A, *params);
  *bytes = ws.peak;
  return COLAGB_OK;
}

extern "C" int colagb_cg_batched_csr_solve(const colagb_batched_csr* A, const double* B, double* X,
                                           const colagb_ir_params* params, int32_t* per_system_iters,
                                           int32_t* per_system_status, double* relres, void* workspace,
                                           size_t workspace_bytes, colagb_ir_result* result, void* stream) {
  COLAGB_TRY(validate_batched(A, params));
  if (!result) return fail(COLAGB_ERR_INVALID, "batched CG: null result");
  const int64_t S_all = A->num_systems;
  result->sweeps = 0;
  result->total_inner_iters = 0;
  result->status = COLAGB_OK;
  result->schedule = params->schedule;
  result->companion_systems = 0;
  if (S_all == 0 || A->n == 0) return COLAGB_OK;
  if (!B || !X) return fail(COLAGB_ERR_INVALID, "batched CG: null B/X");
  if (A->n % 4 != 0 || (uintptr_t)B % 16 != 0 || (uintptr_t)X % 16 != 0)
    return fail(COLAGB_ERR_INVALID, "batched CG: n must be a multiple of 4 and B, X 16-byte aligned");
  Bump ws(workspace, workspace_bytes);
  BatchedWs w = carve_batched(ws, *A, *params);
  if (workspace == nullptr || ws.overflow())
    return fail(COLAGB_ERR_WORKSPACE, "batched CG: workspace too small (need " + std::to_string(ws.peak) + ")");
  cudaStream_t st = as_stream(stream);
  if (use_block(*A, *params)) {
    result->schedule = COLAGB_SCHED_BLOCK;
    int mx = 0;
    COLAGB_TRY(block_pcg_solve(A, B, X, params, per_system_iters, per_system_status, relres, w.block, w.block_bytes,
                               &mx, st));
    result->sweeps = mx;
    return COLAGB_OK;
  }
  const int csize = pick_cluster(*params, A->n);
  const bool try_onchip = params->matvec == COLAGB_MATVEC_FP32 &&
                          (params->schedule == COLAGB_SCHED_AUTO || params->schedule == COLAGB_SCHED_ONCHIP);
  for (int64_t s0 = 0; s0 < S_all; s0 += kMaxBatch) {
    const int64_t S = (S_all - s0) < kMaxBatch ? (S_all - s0) : kMaxBatch;
    colagb_batched_csr sub = *A;
    sub.num_systems = S;
    sub.values = A->values + (A->shared_values ? 0 : s0 * A->nnz);
    sub.g_values = A->g_values ? A->g_values + s0 * A->g_nnz : nullptr;
    bool used = false;
    unsigned int* comp = nullptr;
    if (try_onchip)
      COLAGB_TRY(onchip_pcg_solve(&sub, B + s0 * A->n, X + s0 * A->n, params,
                                  per_system_iters ? per_system_iters + s0 : nullptr,
                                  per_system_status ? per_system_status + s0 : nullptr, relres ? relres + s0 : nullptr,
                                  w.nrep, w.onchip, w.onchip_bytes, &used, &comp, st));
    if (!used && params->schedule == COLAGB_SCHED_ONCHIP)
      return fail(COLAGB_ERR_UNSUPPORTED,
                  "batched CG: the on-chip schedule needs a pattern of at most 9 diagonals (FSAI: G lower "
                  "triangular, at most 5 diagonals) and p, r, d of one system within the shared memory of a "
                  "16-CTA cluster");
    result->schedule = used ? COLAGB_SCHED_ONCHIP
                            : csize == 16 ? COLAGB_SCHED_CLUSTER16 : csize == 8 ? COLAGB_SCHED_CLUSTER8 : COLAGB_SCHED_GRID;
    if (used || csize > 0) {
      if (!used)
        COLAGB_TRY(cluster_pcg_solve(&sub, B + s0 * A->n, X + s0 * A->n, params,
                                     per_system_iters ? per_system_iters + s0 : nullptr,
                                     per_system_status ? per_system_status + s0 : nullptr,
                                     relres ? relres + s0 : nullptr, w.r, w.p, w.ap, w.d, w.z, w.t, w.dinv, w.nrep,
                                     csize, w.v16, w.dg16, st));
      if (params->no_wait) {
        result->sweeps = -1;
        result->companion_systems = -1;
        continue;
      }
      int mx[2] = {0, 0};
      std::vector<int> hrep(S);
      unsigned int hcomp = 0;
      COLAGB_CUDA(cudaMemcpyAsync(hrep.data(), w.nrep, S * sizeof(int), cudaMemcpyDeviceToHost, st));
      if (used && comp)
        COLAGB_CUDA(cudaMemcpyAsync(&hcomp, comp, sizeof(unsigned int), cudaMemcpyDeviceToHost, st));
      COLAGB_CUDA(cudaStreamSynchronize(st));
      result->companion_systems += (int32_t)hcomp;
      for (int64_t q = 0; q < S; ++q) mx[0] = hrep[q] > mx[0] ? hrep[q] : mx[0];
      result->sweeps = mx[0] > result->sweeps ? mx[0] : result->sweeps;
      continue;
    }
    BatchedArgs a;
    a.n = A->n;
    a.nnz = A->nnz;
    a.S = S;
    a.indptr = A->indptr;
    a.indices = A->indices;
    a.vstride = A->shared_values ? 0 : A->nnz;
    a.vals = A->values + s0 * a.vstride;
    a.g_nnz = A->g_nnz;
    a.g_indptr = A->g_indptr;
    a.g_indices = A->g_indices;
    a.gt_indptr = A->gt_indptr;
    a.gt_indices = A->gt_indices;
    a.gt_perm = A->gt_perm;
    a.g_vals = A->g_values ? A->g_values + s0 * A->g_nnz : nullptr;
    a.B = B + s0 * A->n;
    a.X = X + s0 * A->n;
    a.r = w.r; a.p = w.p; a.ap = w.ap; a.d = w.d; a.z = w.z; a.t = w.t; a.dinv = w.dinv;
    a.acc = w.acc;
    a.bnorm = w.bnorm;
    a.out_status = per_system_status ? per_system_status + s0 : nullptr;
    a.out_iters = per_system_iters ? per_system_iters + s0 : nullptr;
    a.out_relres = relres ? relres + s0 : nullptr;
    a.summary = w.summary;
    a.tol = params->tol;
    a.inner_tol = params->inner_tol;
    a.max_sweeps = params->max_sweeps;
    a.max_inner = params->max_inner_iters;
    a.prec_kind = params->preconditioner;
    a.fallback = params->fallback;
    a.mode = params->mode;
    a.gb.count = w.bar;
    a.gb.generation = w.bar + 1;
    a.gb.err = reinterpret_cast<int*>(w.bar + 2);
    a.gb.spin_limit = params->spin_limit > 0 ? params->spin_limit : kDefaultSpinLimit;
    const size_t smem = batched_smem(S);
    if (smem > 48 * 1024)
      COLAGB_CUDA(cudaFuncSetAttribute(k_batched_ir, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int occ = 0;
    COLAGB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_batched_ir, kThreads, smem));
    if (occ < 1) return fail(COLAGB_ERR_UNSUPPORTED, "batched CG kernel cannot be resident");
    const int nb = num_sms() * (occ < 8 ? occ : 8);
    a.gb.nblocks = (unsigned)nb;
    COLAGB_CUDA(cudaMemsetAsync(w.bar, 0, 8 * sizeof(unsigned int), st));
    COLAGB_CUDA(cudaMemsetAsync(w.acc, 0, 6 * S * sizeof(double), st));
    void* args[] = {&a};
    COLAGB_CUDA(cudaLaunchCooperativeKernel((const void*)k_batched_ir, dim3(nb), dim3(kThreads), args, smem, st));
    int h[2] = {0, 0};
    unsigned int herr = 0;
    COLAGB_CUDA(cudaMemcpyAsync(h, w.summary, 2 * sizeof(int), cudaMemcpyDeviceToHost, st));
    COLAGB_CUDA(cudaMemcpyAsync(&herr, w.bar + 2, sizeof(unsigned int), cudaMemcpyDeviceToHost, st));
    COLAGB_CUDA(cudaStreamSynchronize(st));
    if (herr != 0) {
      result->status = COLAGB_ERR_TIMEOUT;
      return fail(COLAGB_ERR_TIMEOUT, "batched CG: a grid barrier timed out");
    }
    result->sweeps = h[0] > result->sweeps ? h[0] : result->sweeps;
    result->total_inner_iters = h[1] > result->total_inner_iters ? h[1] : result->total_inner_iters;
  }
  return COLAGB_OK;
}
