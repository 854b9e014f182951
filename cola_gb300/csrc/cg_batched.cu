// Batched independent SPD systems sharing one CSR sparsity pattern, solved to a true FP64 relative
// residual by FP32 preconditioned CG inside FP64 iterative refinement -- one persistent launch.
//
// Per system s (the reference runs one cola.linalg.solve(PSD(Sparse), b, CG(P=...)) per system,
// cola/linalg/inverse/inv.py:66-69 -> cg.py:94-154; the inner loop below is that PCG step):
//   x = 0, r64 = b
//   sweep: rhat = r64 / |r64| (FP32) ; d = PCG_fp32(A, rhat) to |r_inner| <= inner_tol
//          x += |r64| d (FP64) ; r64 = b - A x (FP64, from the FP32 stored values) ; relres = |r64| / |b|
//   until relres <= tol.
// Preconditioners: none, Jacobi (CG(P=Diagonal(1/diag A))), FSAI (P = G^T G, G lower triangular
// on A's lower pattern).  The FP64 true residual is the judge: a system whose FSAI sweep fails to
// halve its true residual continues with Jacobi (status COLAGB_SYS_FALLBACK).
//
// Work distribution: every phase splits the currently active systems into q row chunks each
// (q*nact ~ 8 chunks per CTA) and deals chunks round-robin over the co-resident CTAs, so CTAs
// stay busy as systems converge.  Per-system sums are CTA-reduced and added to FP64 accumulators.
#include <string>

#include "common.cuh"

namespace colagb {

constexpr int kMaxBatch = 1024;  // systems per launch (host splits larger batches)

struct BatchedArgs {
  int64_t n, nnz, S;
  const int32_t* indptr;
  const int32_t* indices;
  const float* vals;
  int64_t g_nnz;
  const int32_t* g_indptr;
  const int32_t* g_indices;
  const int32_t* gt_indptr;
  const int32_t* gt_indices;
  const int32_t* gt_perm;
  const float* g_vals;
  const double* B;
  double* X;
  float *r, *p, *ap, *d, *z, *t, *dinv;  // [S][n]
  double* r64;                           // [S][n]
  double* acc;                           // [6][S]
  double* bnorm;                         // [S]
  int* out_status;                       // [S] (may be null)
  int* out_iters;                        // [S] (may be null)
  double* out_relres;                    // [S] (may be null)
  int* summary;                          // [4]: sweeps, max total inner iters, -, -
  double tol, inner_tol;
  int max_sweeps, max_inner, prec_kind, fallback;
  GridBarrier gb;
};

struct BatchedSmem {
  int* act;        // active system list
  double* gamma;   // <r, z>
  float* alpha;
  float* beta;
  double* rn64;    // |r64|
  double* relres;
  int* prec;       // per-system preconditioner kind
  int* status;     // COLAGB_SYS_*
  int* inner_on;   // inner CG still running
  int* it_sweep;   // inner iterations this sweep
  int* it_total;   // inner iterations over all sweeps
  float* rnin;     // inner |r|
};

__device__ __forceinline__ void chunking(int nact, int nb, int64_t n, int& q, int64_t& cs) {
  const int target = 8 * nb;
  q = nact > 0 ? (target + nact - 1) / nact : 1;
  if (q < 1) q = 1;
  if ((int64_t)q > n) q = (int)n;
  cs = (n + q - 1) / q;
}

// f(s, i) -> float contribution, summed per system into acc_s[s] (FP64 atomics, one per chunk).
// If acc_s is null, f is evaluated for its side effects only.
template <class F>
__device__ __forceinline__ void sweep_chunks(const int* act, int nact, int64_t n, double* acc_s, F f,
                                             float* red) {
  int q;
  int64_t cs;
  chunking(nact, gridDim.x, n, q, cs);
  const int total = nact * q;
  for (int ch = blockIdx.x; ch < total; ch += gridDim.x) {
    const int s = act[ch / q];
    const int64_t i0 = (int64_t)(ch % q) * cs;
    const int64_t i1 = (i0 + cs < n) ? i0 + cs : n;
    float v = 0.f;
    for (int64_t i = i0 + threadIdx.x; i < i1; i += blockDim.x) v += f(s, i);
    if (acc_s) {
      v = block_sum(v, red);
      if (threadIdx.x == 0) atomicAdd(acc_s + s, (double)v);
    }
  }
}

template <class F>
__device__ __forceinline__ void sweep_chunks64(const int* act, int nact, int64_t n, double* acc_s, F f,
                                               double* red) {
  int q;
  int64_t cs;
  chunking(nact, gridDim.x, n, q, cs);
  const int total = nact * q;
  for (int ch = blockIdx.x; ch < total; ch += gridDim.x) {
    const int s = act[ch / q];
    const int64_t i0 = (int64_t)(ch % q) * cs;
    const int64_t i1 = (i0 + cs < n) ? i0 + cs : n;
    double v = 0.0;
    for (int64_t i = i0 + threadIdx.x; i < i1; i += blockDim.x) v += f(s, i);
    v = block_sum(v, red);
    if (threadIdx.x == 0) atomicAdd(acc_s + s, v);
  }
}

// Rebuild the active list from a predicate (identical in every CTA).
template <class P>
__device__ __forceinline__ int build_active(int S, int* act, P pred) {
  __shared__ int s_n;
  __syncthreads();
  if (threadIdx.x == 0) {
    int c = 0;
    for (int s = 0; s < S; ++s)
      if (pred(s)) act[c++] = s;
    s_n = c;
  }
  __syncthreads();
  const int r = s_n;
  __syncthreads();
  return r;
}

__device__ __forceinline__ float csr_row(const BatchedArgs& a, int s, int64_t i, const float* v) {
  const float* vals = a.vals + (int64_t)s * a.nnz;
  const float* vs = v + (int64_t)s * a.n;
  const int32_t b = a.indptr[i], e = a.indptr[i + 1];
  float acc = 0.f;
  for (int32_t j = b; j < e; ++j) acc += vals[j] * vs[a.indices[j]];
  return acc;
}

__global__ void __launch_bounds__(256) k_batched_ir(BatchedArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int S = (int)a.S;
  const int64_t n = a.n;
  BatchedSmem m;
  {
    unsigned char* q = smem_raw;
    auto takeb = [&](size_t bytes) { unsigned char* r = q; q += (bytes + 15) / 16 * 16; return r; };
    m.gamma = reinterpret_cast<double*>(takeb(sizeof(double) * S));
    m.rn64 = reinterpret_cast<double*>(takeb(sizeof(double) * S));
    m.relres = reinterpret_cast<double*>(takeb(sizeof(double) * S));
    m.act = reinterpret_cast<int*>(takeb(sizeof(int) * S));
    m.alpha = reinterpret_cast<float*>(takeb(sizeof(float) * S));
    m.beta = reinterpret_cast<float*>(takeb(sizeof(float) * S));
    m.prec = reinterpret_cast<int*>(takeb(sizeof(int) * S));
    m.status = reinterpret_cast<int*>(takeb(sizeof(int) * S));
    m.inner_on = reinterpret_cast<int*>(takeb(sizeof(int) * S));
    m.it_sweep = reinterpret_cast<int*>(takeb(sizeof(int) * S));
    m.it_total = reinterpret_cast<int*>(takeb(sizeof(int) * S));
    m.rnin = reinterpret_cast<float*>(takeb(sizeof(float) * S));
  }
  __shared__ float redf[32];
  __shared__ double redd[32];
  double* acc0 = a.acc;            // |b|^2, later <p, Ap>
  double* acc1 = a.acc + S;        // <r, z>
  double* acc2 = a.acc + 2 * S;    // |r|^2 (inner)
  double* acc3 = a.acc + 3 * S;    // |r64|^2

  // ---------------- setup ----------------
  for (int s = threadIdx.x; s < S; s += blockDim.x) {
    m.prec[s] = a.prec_kind;
    m.status[s] = COLAGB_SYS_RUNNING;
    m.it_total[s] = 0;
  }
  int nact = build_active(S, m.act, [&](int) { return true; });
  // Jacobi diagonal, x = 0, r64 = b, |b|^2
  sweep_chunks64(m.act, nact, n, acc0, [&](int s, int64_t i) -> double {
    const int64_t u = (int64_t)s * n + i;
    if (a.dinv) {
      const float* vals = a.vals + (int64_t)s * a.nnz;
      float dg = 0.f;
      for (int32_t j = a.indptr[i]; j < a.indptr[i + 1]; ++j)
        if (a.indices[j] == i) dg += vals[j];
      a.dinv[u] = dg != 0.f ? 1.f / dg : 1.f;
    }
    const double bv = a.B[u];
    a.X[u] = 0.0;
    a.r64[u] = bv;
    return bv * bv;
  }, redd);
  if (!grid_sync(a.gb)) return;
  for (int s = threadIdx.x; s < S; s += blockDim.x) {
    const double bn = sqrt(__ldcg(acc0 + s));
    m.rn64[s] = bn;
    m.relres[s] = bn > 0.0 ? 1.0 : 0.0;
    if (!(bn > 0.0)) m.status[s] = (bn == 0.0) ? COLAGB_SYS_CONVERGED : COLAGB_SYS_NAN;
    if (blockIdx.x == 0) a.bnorm[s] = bn;
  }
  __syncthreads();
  if (!grid_sync(a.gb)) return;  // every CTA has read acc0
  if (blockIdx.x == 0)
    for (int s = threadIdx.x; s < S; s += blockDim.x) { acc0[s] = 0.0; acc1[s] = 0.0; acc2[s] = 0.0; acc3[s] = 0.0; }
  if (!grid_sync(a.gb)) return;

  int sweep = 0;
  int max_total_inner = 0;
  for (; sweep < a.max_sweeps; ++sweep) {
    // systems needing another sweep
    for (int s = threadIdx.x; s < S; s += blockDim.x)
      if (m.status[s] == COLAGB_SYS_RUNNING && m.relres[s] <= a.tol) m.status[s] = COLAGB_SYS_CONVERGED;
    __syncthreads();
    nact = build_active(S, m.act, [&](int s) { return m.status[s] == COLAGB_SYS_RUNNING; });
    if (nact == 0) break;
    bool any_fsai = false;
    for (int j = 0; j < nact; ++j) any_fsai |= (m.prec[m.act[j]] == COLAGB_PREC_FSAI);

    // ---- inner init: r = r64/|r64|, d = 0 ----
    sweep_chunks(m.act, nact, n, nullptr, [&](int s, int64_t i) -> float {
      const int64_t u = (int64_t)s * n + i;
      a.r[u] = (float)(a.r64[u] / m.rn64[s]);
      a.d[u] = 0.f;
      return 0.f;
    }, redf);
    if (!grid_sync(a.gb)) return;
    if (any_fsai) {
      sweep_chunks(m.act, nact, n, nullptr, [&](int s, int64_t i) -> float {
        if (m.prec[s] != COLAGB_PREC_FSAI) return 0.f;
        const float* g = a.g_vals + (int64_t)s * a.g_nnz;
        const float* rs = a.r + (int64_t)s * n;
        float v = 0.f;
        for (int32_t e = a.g_indptr[i]; e < a.g_indptr[i + 1]; ++e) v += g[e] * rs[a.g_indices[e]];
        a.t[(int64_t)s * n + i] = v;
        return 0.f;
      }, redf);
      if (!grid_sync(a.gb)) return;
    }
    // z = M r ; p = z ; <r, z>, |r|^2
    auto apply_m = [&](int s, int64_t i) -> float {
      const int64_t u = (int64_t)s * n + i;
      const int pk = m.prec[s];
      if (pk == COLAGB_PREC_JACOBI) return a.dinv[u] * a.r[u];
      if (pk == COLAGB_PREC_FSAI) {
        const float* g = a.g_vals + (int64_t)s * a.g_nnz;
        const float* ts = a.t + (int64_t)s * n;
        float v = 0.f;
        for (int32_t e = a.gt_indptr[i]; e < a.gt_indptr[i + 1]; ++e) v += g[a.gt_perm[e]] * ts[a.gt_indices[e]];
        return v;
      }
      return a.r[u];
    };
    sweep_chunks(m.act, nact, n, acc1, [&](int s, int64_t i) -> float {
      const int64_t u = (int64_t)s * n + i;
      const float zv = apply_m(s, i);
      if (a.z) a.z[u] = zv;
      a.p[u] = zv;
      return a.r[u] * zv;
    }, redf);
    sweep_chunks(m.act, nact, n, acc2, [&](int s, int64_t i) -> float {
      const float rv = a.r[(int64_t)s * n + i];
      return rv * rv;
    }, redf);
    if (!grid_sync(a.gb)) return;
    for (int s = threadIdx.x; s < S; s += blockDim.x) {
      m.inner_on[s] = 0;
      m.it_sweep[s] = 0;
    }
    __syncthreads();
    for (int j = threadIdx.x; j < nact; j += blockDim.x) {
      const int s = m.act[j];
      m.gamma[s] = __ldcg(acc1 + s);
      m.rnin[s] = (float)sqrt(__ldcg(acc2 + s));
      m.inner_on[s] = m.rnin[s] > (float)a.inner_tol && a.max_inner > 0;
    }
    __syncthreads();
    if (!grid_sync(a.gb)) return;
    if (blockIdx.x == 0)
      for (int j = threadIdx.x; j < nact; j += blockDim.x) { acc1[m.act[j]] = 0.0; acc2[m.act[j]] = 0.0; }
    int nin = build_active(S, m.act, [&](int s) { return m.inner_on[s] != 0; });
    if (!grid_sync(a.gb)) return;

    // ---- inner PCG ----
    while (nin > 0) {
      // A: Ap = A p ; <p, Ap>
      sweep_chunks(m.act, nin, n, acc0, [&](int s, int64_t i) -> float {
        const int64_t u = (int64_t)s * n + i;
        const float v = csr_row(a, s, i, a.p);
        a.ap[u] = v;
        return a.p[u] * v;
      }, redf);
      if (!grid_sync(a.gb)) return;
      for (int j = threadIdx.x; j < nin; j += blockDim.x) {
        const int s = m.act[j];
        const double pap = __ldcg(acc0 + s);
        m.alpha[s] = pap > 0.0 ? (float)(m.gamma[s] / pap) : 0.f;
        if (!(pap > 0.0)) {  // breakdown: not SPD in FP32 (or NaN)
          m.inner_on[s] = 0;
          m.status[s] = (pap == pap) ? COLAGB_SYS_BREAKDOWN : COLAGB_SYS_NAN;
        }
      }
      __syncthreads();
      // B: d += alpha p ; r -= alpha Ap ; (no FSAI: <r, z>) ; |r|^2
      sweep_chunks(m.act, nin, n, acc2, [&](int s, int64_t i) -> float {
        const int64_t u = (int64_t)s * n + i;
        const float al = m.alpha[s];
        a.d[u] += al * a.p[u];
        const float rv = a.r[u] - al * a.ap[u];
        a.r[u] = rv;
        return rv * rv;
      }, redf);
      if (!any_fsai) {
        sweep_chunks(m.act, nin, n, acc1, [&](int s, int64_t i) -> float {
          const int64_t u = (int64_t)s * n + i;
          return a.r[u] * apply_m(s, i);
        }, redf);
      }
      if (!grid_sync(a.gb)) return;
      if (any_fsai) {
        // t = G r (FSAI systems) ; then z = G^T t and <r, z> for all systems
        sweep_chunks(m.act, nin, n, nullptr, [&](int s, int64_t i) -> float {
          if (m.prec[s] != COLAGB_PREC_FSAI) return 0.f;
          const float* g = a.g_vals + (int64_t)s * a.g_nnz;
          const float* rs = a.r + (int64_t)s * n;
          float v = 0.f;
          for (int32_t e = a.g_indptr[i]; e < a.g_indptr[i + 1]; ++e) v += g[e] * rs[a.g_indices[e]];
          a.t[(int64_t)s * n + i] = v;
          return 0.f;
        }, redf);
        if (!grid_sync(a.gb)) return;
        sweep_chunks(m.act, nin, n, acc1, [&](int s, int64_t i) -> float {
          const int64_t u = (int64_t)s * n + i;
          const float zv = apply_m(s, i);
          a.z[u] = zv;
          return a.r[u] * zv;
        }, redf);
        if (!grid_sync(a.gb)) return;
      }
      // C: beta, stop tests, p = z + beta p
      for (int j = threadIdx.x; j < nin; j += blockDim.x) {
        const int s = m.act[j];
        const double g1 = __ldcg(acc1 + s);
        const float rn = (float)sqrt(__ldcg(acc2 + s));
        m.beta[s] = m.gamma[s] != 0.0 ? (float)(g1 / m.gamma[s]) : 0.f;
        m.gamma[s] = g1;
        m.rnin[s] = rn;
        m.it_sweep[s] += 1;
        if (!(rn == rn)) { m.inner_on[s] = 0; m.status[s] = COLAGB_SYS_NAN; }
        if (rn <= (float)a.inner_tol || m.it_sweep[s] >= a.max_inner) m.inner_on[s] = 0;
      }
      __syncthreads();
      if (!grid_sync(a.gb)) return;  // all CTAs have read acc0..acc2
      if (blockIdx.x == 0)
        for (int j = threadIdx.x; j < nin; j += blockDim.x) {
          const int s = m.act[j];
          acc0[s] = 0.0; acc1[s] = 0.0; acc2[s] = 0.0;
        }
      nin = build_active(S, m.act, [&](int s) { return m.inner_on[s] != 0; });
      if (nin == 0) break;
      sweep_chunks(m.act, nin, n, nullptr, [&](int s, int64_t i) -> float {
        const int64_t u = (int64_t)s * n + i;
        const float zv = any_fsai ? (a.z ? a.z[u] : 0.f) : apply_m(s, i);
        a.p[u] = zv + m.beta[s] * a.p[u];
        return 0.f;
      }, redf);
      if (!grid_sync(a.gb)) return;
    }

    // ---- refinement: x += |r64| d ; r64 = b - A x ; relres ----
    nact = build_active(S, m.act, [&](int s) { return m.status[s] == COLAGB_SYS_RUNNING; });
    for (int s = threadIdx.x; s < S; s += blockDim.x) {
      m.it_total[s] += m.it_sweep[s];
    }
    __syncthreads();
    {
      int mx = 0;
      for (int s = 0; s < S; ++s) mx = m.it_sweep[s] > mx ? m.it_sweep[s] : mx;
      max_total_inner += mx;
    }
    sweep_chunks(m.act, nact, n, nullptr, [&](int s, int64_t i) -> float {
      const int64_t u = (int64_t)s * n + i;
      a.X[u] += m.rn64[s] * (double)a.d[u];
      return 0.f;
    }, redf);
    if (!grid_sync(a.gb)) return;
    sweep_chunks64(m.act, nact, n, acc3, [&](int s, int64_t i) -> double {
      const int64_t u = (int64_t)s * n + i;
      const float* vals = a.vals + (int64_t)s * a.nnz;
      const double* xs = a.X + (int64_t)s * n;
      double ax = 0.0;
      for (int32_t j = a.indptr[i]; j < a.indptr[i + 1]; ++j) ax += (double)vals[j] * xs[a.indices[j]];
      const double rv = a.B[u] - ax;
      a.r64[u] = rv;
      return rv * rv;
    }, redd);
    if (!grid_sync(a.gb)) return;
    for (int j = threadIdx.x; j < nact; j += blockDim.x) {
      const int s = m.act[j];
      const double rn = sqrt(__ldcg(acc3 + s));
      const double rr = rn / a.bnorm[s];
      if (!(rr == rr)) m.status[s] = COLAGB_SYS_NAN;
      // the FP64 true residual judges the learned preconditioner
      if (a.fallback && m.prec[s] == COLAGB_PREC_FSAI && rr > 0.5 * m.relres[s]) {
        m.prec[s] = COLAGB_PREC_JACOBI;
      }
      m.rn64[s] = rn;
      m.relres[s] = rr;
    }
    __syncthreads();
    if (!grid_sync(a.gb)) return;
    if (blockIdx.x == 0)
      for (int j = threadIdx.x; j < nact; j += blockDim.x) acc3[m.act[j]] = 0.0;
    if (!grid_sync(a.gb)) return;
  }
  // ---- results ----
  if (blockIdx.x == 0) {
    for (int s = threadIdx.x; s < S; s += blockDim.x) {
      int st = m.status[s];
      if (st == COLAGB_SYS_RUNNING) st = m.relres[s] <= a.tol ? COLAGB_SYS_CONVERGED : COLAGB_SYS_MAX_ITERS;
      if (st == COLAGB_SYS_CONVERGED && a.prec_kind == COLAGB_PREC_FSAI && m.prec[s] != COLAGB_PREC_FSAI)
        st = COLAGB_SYS_FALLBACK;
      if (a.out_status) a.out_status[s] = st;
      if (a.out_iters) a.out_iters[s] = m.it_total[s];
      if (a.out_relres) a.out_relres[s] = m.relres[s];
    }
    if (threadIdx.x == 0) {
      a.summary[0] = sweep;
      a.summary[1] = max_total_inner;
    }
  }
}

static size_t batched_smem(int64_t S) { return (size_t)S * (3 * 8 + 9 * 4) + 16 * 12; }

struct BatchedWs {
  float *r, *p, *ap, *d, *z, *t, *dinv;
  double *r64, *acc, *bnorm;
  unsigned int* bar;  // count, generation, err
  int* summary;
};

static BatchedWs carve_batched(Bump& ws, const colagb_batched_csr& A, const colagb_ir_params& prm) {
  const int64_t S = A.num_systems < kMaxBatch ? A.num_systems : kMaxBatch;
  const int64_t sn = S * A.n;
  BatchedWs w;
  w.r = ws.take<float>(sn);
  w.p = ws.take<float>(sn);
  w.ap = ws.take<float>(sn);
  w.d = ws.take<float>(sn);
  const bool fsai = prm.preconditioner == COLAGB_PREC_FSAI;
  const bool jac = prm.preconditioner == COLAGB_PREC_JACOBI || (fsai && prm.fallback);
  w.z = fsai ? ws.take<float>(sn) : nullptr;
  w.t = fsai ? ws.take<float>(sn) : nullptr;
  w.dinv = jac ? ws.take<float>(sn) : nullptr;
  w.r64 = ws.take<double>(sn);
  w.acc = ws.take<double>(6 * S);
  w.bnorm = ws.take<double>(S);
  w.bar = ws.take<unsigned int>(8);
  w.summary = ws.take<int>(8);
  return w;
}

static int validate_batched(const colagb_batched_csr* A, const colagb_ir_params* prm) {
  if (!A || !prm) return fail(COLAGB_ERR_INVALID, "batched CG: null argument");
  if (A->n < 0 || A->nnz < 0 || A->num_systems < 0) return fail(COLAGB_ERR_INVALID, "batched CG: negative size");
  if (A->n > 0 && (!A->indptr || (A->nnz > 0 && (!A->indices || !A->values))))
    return fail(COLAGB_ERR_INVALID, "batched CG: missing CSR arrays");
  if (prm->preconditioner < 0 || prm->preconditioner > 2)
    return fail(COLAGB_ERR_INVALID, "batched CG: unknown preconditioner");
  if (prm->preconditioner == COLAGB_PREC_FSAI &&
      (!A->g_indptr || !A->g_indices || !A->gt_indptr || !A->gt_indices || !A->gt_perm || !A->g_values))
    return fail(COLAGB_ERR_INVALID, "batched CG: FSAI preconditioner needs G and G^T patterns and values");
  if (!(prm->tol > 0) || !(prm->inner_tol > 0)) return fail(COLAGB_ERR_INVALID, "batched CG: tolerances must be > 0");
  if (prm->max_sweeps < 0 || prm->max_inner_iters < 0) return fail(COLAGB_ERR_INVALID, "batched CG: negative limits");
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
  Bump ws(nullptr, 0);
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
  if (S_all == 0 || A->n == 0) return COLAGB_OK;
  if (!B || !X) return fail(COLAGB_ERR_INVALID, "batched CG: null B/X");
  Bump ws(workspace, workspace_bytes);
  BatchedWs w = carve_batched(ws, *A, *params);
  if (workspace == nullptr || ws.overflow())
    return fail(COLAGB_ERR_WORKSPACE, "batched CG: workspace too small (need " + std::to_string(ws.peak) + ")");
  cudaStream_t st = as_stream(stream);
  for (int64_t s0 = 0; s0 < S_all; s0 += kMaxBatch) {
    const int64_t S = (S_all - s0) < kMaxBatch ? (S_all - s0) : kMaxBatch;
    BatchedArgs a;
    a.n = A->n;
    a.nnz = A->nnz;
    a.S = S;
    a.indptr = A->indptr;
    a.indices = A->indices;
    a.vals = A->values + s0 * A->nnz;
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
    a.r64 = w.r64;
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
    a.gb.count = w.bar;
    a.gb.generation = w.bar + 1;
    a.gb.err = reinterpret_cast<int*>(w.bar + 2);
    a.gb.spin_limit = params->spin_limit > 0 ? params->spin_limit : kDefaultSpinLimit;
    const size_t smem = batched_smem(S);
    if (smem > 48 * 1024)
      COLAGB_CUDA(cudaFuncSetAttribute(k_batched_ir, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int occ = 0;
    COLAGB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_batched_ir, 256, smem));
    if (occ < 1) return fail(COLAGB_ERR_UNSUPPORTED, "batched CG kernel cannot be resident");
    const int nb = num_sms() * (occ < 4 ? occ : 4);
    a.gb.nblocks = (unsigned)nb;
    COLAGB_CUDA(cudaMemsetAsync(w.bar, 0, 8 * sizeof(unsigned int), st));
    COLAGB_CUDA(cudaMemsetAsync(w.acc, 0, 6 * S * sizeof(double), st));
    void* args[] = {&a};
    COLAGB_CUDA(cudaLaunchCooperativeKernel((const void*)k_batched_ir, dim3(nb), dim3(256), args, smem, st));
    int h[4] = {0, 0, 0, 0};
    unsigned int herr = 0;
    COLAGB_CUDA(cudaMemcpyAsync(h, w.summary, 2 * sizeof(int), cudaMemcpyDeviceToHost, st));
    COLAGB_CUDA(cudaMemcpyAsync(&herr, w.bar + 2, sizeof(unsigned int), cudaMemcpyDeviceToHost, st));
    COLAGB_CUDA(cudaStreamSynchronize(st));
    if (herr != 0) {
      result->status = COLAGB_ERR_TIMEOUT;
      return fail(COLAGB_ERR_TIMEOUT, "batched CG: a grid barrier timed out");
    }
    result->sweeps = h[0] > result->sweeps ? h[0] : result->sweeps;
    result->total_inner_iters += h[1];
  }
  return COLAGB_OK;
}
