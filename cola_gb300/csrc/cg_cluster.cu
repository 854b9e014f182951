// Batched shared-pattern PCG, one thread-block cluster per system.
//
// Same algorithm as k_batched_ir (cg_batched.cu: FP32 preconditioned CG, FP64 solution, FP64 residual
// replacement, Jacobi / FSAI / learned-FSAI preconditioners, the FP64 true residual as the only
// convergence test and as the judge of the learned factor) but scheduled the sm_103a way:
//   * the grid holds one cluster of kCL CTAs per system; clusters are independent, so the hardware
//     starts a new system's cluster as soon as one finishes (dynamic load balance, no grid-wide sync);
//   * each CTA owns a fixed contiguous row range of its system for the whole solve;
//   * phase boundaries are hardware cluster barriers (barrier.cluster arrive/wait via
//     cooperative_groups); the per-step dot products are FP32 block sums exchanged through
//     distributed shared memory and combined by the same butterfly in every CTA, so every CTA of a
//     cluster derives bit-identical alpha / beta (|b| and the FP64 true residual stay FP64);
//   * with ~10-19 systems in flight their vectors and values (~10 MB per 512^2 system) largely stay
//     in the 126 MB L2 across iterations.
#include <cooperative_groups.h>

#include <algorithm>
#include <string>

#include "cluster.cuh"
#include "common.cuh"

namespace cg = cooperative_groups;

namespace colagb {

constexpr int kCT = 1024;  // threads per CTA

struct ClusterArgs {
  int64_t n, nnz, S, vstride;
  const int32_t* __restrict__ indptr;
  const int32_t* __restrict__ indices;
  const float* __restrict__ vals;
  // BF16 inner matvec: off-diagonal values in BF16 (diagonal slots zero) and the consistent FP32
  // diagonal, one array per value set (stride vstride / n, 0 for shared values)
  const __nv_bfloat16* __restrict__ v16;
  const float* __restrict__ dg16;
  int64_t dstride;
  int64_t g_nnz;
  const int32_t* g_indptr;
  const int32_t* g_indices;
  const int32_t* gt_indptr;
  const int32_t* gt_indices;
  const int32_t* gt_perm;
  const float* g_vals;
  const double* B;
  double* X;
  float *r, *p, *ap, *d, *z, *t, *dinv;
  int* out_status;
  int* out_iters;
  double* out_relres;
  int* out_nrep;
  double tol, inner_tol;
  int max_sweeps, max_inner, prec_kind, fallback, mode;
};

// `x` (the search direction) is rewritten by the other CTAs of the cluster during the kernel: no
// __restrict__, so it is never read through the non-coherent read-only cache.
__device__ __forceinline__ float row_dot_f(const ClusterArgs& a, const float* __restrict__ vals, const float* x,
                                           int64_t i) {
  const int32_t b = __ldg(a.indptr + i), e = __ldg(a.indptr + i + 1);
  float acc = 0.f;
#pragma unroll
  for (int k = 0; k < 6; ++k)
    if (b + k < e) acc += vals[b + k] * x[__ldg(a.indices + b + k)];
  for (int32_t j = b + 6; j < e; ++j) acc += vals[j] * x[__ldg(a.indices + j)];
  return acc;
}

// BF16 form: A' x at row i = d'_i x_i + sum_j bf16(a_ij) x_j (the diagonal slot of v16 holds zero).
__device__ __forceinline__ float row_dot_b(const ClusterArgs& a, const __nv_bfloat16* __restrict__ v16,
                                          const float* __restrict__ dg, const float* x, int64_t i) {
  const int32_t b = __ldg(a.indptr + i), e = __ldg(a.indptr + i + 1);
  float acc = dg[i] * x[i];
#pragma unroll
  for (int k = 0; k < 6; ++k)
    if (b + k < e) acc += __bfloat162float(v16[b + k]) * x[__ldg(a.indices + b + k)];
  for (int32_t j = b + 6; j < e; ++j) acc += __bfloat162float(v16[j]) * x[__ldg(a.indices + j)];
  return acc;
}

// One value set per block row: v16 / dg16 from FP32 CSR values (see COLAGB_MATVEC_BF16).
__global__ void k_bf16_consistent(const int32_t* __restrict__ indptr, const int32_t* __restrict__ indices,
                                  const float* __restrict__ vals, int64_t n, int64_t nnz,
                                  __nv_bfloat16* __restrict__ v16, float* __restrict__ dg16) {
  const int64_t s = blockIdx.y;
  vals += s * nnz;
  v16 += s * nnz;
  dg16 += s * n;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double d = 0.0, corr = 0.0;
    for (int32_t j = indptr[i]; j < indptr[i + 1]; ++j) {
      const float v = vals[j];
      if (indices[j] == i) {
        d += (double)v;
        v16[j] = __float2bfloat16_rn(0.f);
      } else {
        const __nv_bfloat16 h = __float2bfloat16_rn(v);
        v16[j] = h;
        corr += (double)__bfloat162float(h) - (double)v;
      }
    }
    dg16[i] = (float)(d - corr);
  }
}

template <int CL, bool BF>
__global__ void __launch_bounds__(kCT, 1) k_cluster_pcg(const __grid_constant__ ClusterArgs a) {
  cg::cluster_group cl = cg::this_cluster();
  const int rank = (int)cl.block_rank();
  const int64_t s = blockIdx.x / CL;
  if (s >= a.S) return;  // whole clusters only (grid = S * CL)
  __shared__ double slots[2][8];
  __shared__ double red[32];
  __shared__ double bcast[8];
  __shared__ float fslots[2][2 * CL];  // cluster_sum_f slots: NQ <= 2 sums x CL ranks
  __shared__ float wpart[2 * 32];
  int buf = 0, fbuf = 0;
  auto next_slot = [&]() { double* p = slots[buf]; buf ^= 1; return p; };
  auto next_fslot = [&]() { float* p = fslots[fbuf]; fbuf ^= 1; return p; };

  const int64_t n = a.n;
  const int64_t rows = ((n + CL - 1) / CL + 3) / 4 * 4;
  const int64_t i0 = rank * rows < n ? rank * rows : n;
  const int64_t i1 = (rank + 1) * rows < n ? (rank + 1) * rows : n;
  const int64_t so = s * n;
  const float* __restrict__ vals = a.vals + s * a.vstride;
  const __nv_bfloat16* __restrict__ v16 = BF ? a.v16 + s * a.vstride : nullptr;
  const float* __restrict__ dg16 = BF ? a.dg16 + s * a.dstride : nullptr;
  // vectors written by several CTAs of the cluster: plain pointers (see row_dot_f)
  float* r = a.r + so;
  float* p = a.p + so;
  float* ap = a.ap + so;
  float* d = a.d + so;
  float* z = a.z + so;
  float* dinv = a.dinv ? a.dinv + so : nullptr;
  double* X = a.X + so;
  const double* __restrict__ B = a.B + so;
  const float* g = a.g_vals ? a.g_vals + s * a.g_nnz : nullptr;
  float* t = a.t ? a.t + so : nullptr;
  const int tid = threadIdx.x;
  const int64_t v0 = i0 + 4 * (int64_t)tid;  // first float4 group of this thread
  const int64_t vstep = 4 * (int64_t)kCT;

  int prec = a.prec_kind;
  // ---- setup: |b|^2, x = 0, d = 0, Jacobi diagonal ----
  double v1[1] = {0.0};
  for (int64_t i = i0 + tid; i < i1; i += kCT) {
    const double bv = B[i];
    v1[0] += bv * bv;
    X[i] = 0.0;
    d[i] = 0.f;
    if (dinv) {
      float dg = 0.f;
      for (int32_t j = a.indptr[i]; j < a.indptr[i + 1]; ++j)
        if (a.indices[j] == i) dg += vals[j];
      dinv[i] = dg != 0.f ? 1.f / dg : 1.f;
    }
  }
  cluster_sum<1, CL>(cl, v1, next_slot(), red, bcast);
  const double bnorm = sqrt(v1[0]);
  int status = COLAGB_SYS_RUNNING;
  double relres = bnorm > 0.0 ? 1.0 : 0.0;
  if (!(bnorm > 0.0)) status = bnorm == 0.0 ? COLAGB_SYS_CONVERGED : COLAGB_SYS_NAN;
  const double binv = bnorm > 0.0 ? 1.0 / bnorm : 1.0;

  // r = b/|b| - A x (x = 0) in FP64 ; |r|^2 ; <r, M r>
  auto residual = [&](double (&q)[2]) {
    q[0] = q[1] = 0.0;
    for (int64_t i = i0 + tid; i < i1; i += kCT) {
      const int32_t b0 = a.indptr[i], e0 = a.indptr[i + 1];
      double ax = 0.0;
      for (int32_t j = b0; j < e0; ++j) ax += (double)vals[j] * X[a.indices[j]];
      const double rv = B[i] * binv - ax;
      const float rf = (float)rv;
      r[i] = rf;
      q[0] += rv * rv;
      q[1] += (double)(rf * ((prec == COLAGB_PREC_JACOBI ? dinv[i] : 1.f) * rf));
    }
  };
  // t = G r (FSAI)
  auto fsai_t = [&]() {
    for (int64_t i = i0 + tid; i < i1; i += kCT) {
      float v = 0.f;
      for (int32_t e = a.g_indptr[i]; e < a.g_indptr[i + 1]; ++e) v += g[e] * r[a.g_indices[e]];
      t[i] = v;
    }
  };
  // z = M r, <r, z>
  auto apply_z = [&](float (&q)[1]) {
    float qf = 0.f;
    for (int64_t i = i0 + tid; i < i1; i += kCT) {
      float zv;
      if (prec == COLAGB_PREC_FSAI) {
        float v = 0.f;
        for (int32_t e = a.gt_indptr[i]; e < a.gt_indptr[i + 1]; ++e) v += g[a.gt_perm[e]] * t[a.gt_indices[e]];
        zv = v;
      } else {
        zv = prec == COLAGB_PREC_JACOBI ? dinv[i] * r[i] : r[i];
      }
      z[i] = zv;
      qf += r[i] * zv;
    }
    q[0] = qf;
  };

  cl.sync();  // x, d zero and bnorm known everywhere before the residual reads x
  double q2[2];
  residual(q2);
  cluster_sum<2, CL>(cl, q2, next_slot(), red, bcast);
  float rn = (float)sqrt(q2[0]);
  float rmax = rn;
  double relres_prev = relres;
  if (status == COLAGB_SYS_RUNNING && prec == COLAGB_PREC_FSAI) {
    fsai_t();
    cl.sync();
  }
  float q1[1];
  apply_z(q1);
  cluster_sum_f<1, CL>(cl, q1, wpart, next_fslot());
  float gamma = q1[0];
  if (status == COLAGB_SYS_RUNNING && rn <= (float)a.tol) status = COLAGB_SYS_CONVERGED;
  for (int64_t i = i0 + tid; i < i1; i += kCT) p[i] = z[i];
  cl.sync();

  int it = 0, nrep = 0, it_rep = 0;
  const float delta = (float)a.inner_tol;
  while (status == COLAGB_SYS_RUNNING) {
    // A: Ap = A p ; <p, Ap>
    float qaf = 0.f;
    for (int64_t i = i0 + tid; i < i1; i += 2 * kCT) {
      const int64_t i2 = i + kCT;
      float y0, y1;
      if constexpr (BF) {
        y0 = row_dot_b(a, v16, dg16, p, i);
        y1 = i2 < i1 ? row_dot_b(a, v16, dg16, p, i2) : 0.f;
      } else {
        y0 = row_dot_f(a, vals, p, i);
        y1 = i2 < i1 ? row_dot_f(a, vals, p, i2) : 0.f;
      }
      ap[i] = y0;
      float acc = p[i] * y0;
      if (i2 < i1) {
        ap[i2] = y1;
        acc += p[i2] * y1;
      }
      qaf += acc;
    }
    float qa[1] = {qaf};
    cluster_sum_f<1, CL>(cl, qa, wpart, next_fslot());
    const float pap = qa[0];
    if (!(pap > 0.f)) {  // not SPD in FP32 (or NaN)
      status = (pap == pap) ? COLAGB_SYS_BREAKDOWN : COLAGB_SYS_NAN;
      break;
    }
    const float alpha = gamma / pap;
    // B: d += alpha p ; r -= alpha Ap ; |r|^2 ; <r, M r>  (own rows, 128-bit)
    float qb0 = 0.f, qb1 = 0.f;
    for (int64_t i = v0; i < i1; i += vstep) {
      if (i + 3 < i1) {
        const float4 dv = *reinterpret_cast<const float4*>(d + i);
        const float4 pv = *reinterpret_cast<const float4*>(p + i);
        const float4 rv = *reinterpret_cast<const float4*>(r + i);
        const float4 av = *reinterpret_cast<const float4*>(ap + i);
        const float4 di = prec == COLAGB_PREC_JACOBI ? *reinterpret_cast<const float4*>(dinv + i)
                                                     : make_float4(1.f, 1.f, 1.f, 1.f);
        float4 dn, rnv;
        dn.x = dv.x + alpha * pv.x; dn.y = dv.y + alpha * pv.y; dn.z = dv.z + alpha * pv.z; dn.w = dv.w + alpha * pv.w;
        rnv.x = rv.x - alpha * av.x; rnv.y = rv.y - alpha * av.y; rnv.z = rv.z - alpha * av.z; rnv.w = rv.w - alpha * av.w;
        *reinterpret_cast<float4*>(d + i) = dn;
        *reinterpret_cast<float4*>(r + i) = rnv;
        qb0 += rnv.x * rnv.x + rnv.y * rnv.y + rnv.z * rnv.z + rnv.w * rnv.w;
        qb1 += rnv.x * di.x * rnv.x + rnv.y * di.y * rnv.y + rnv.z * di.z * rnv.z + rnv.w * di.w * rnv.w;
      } else {
        for (int64_t k = i; k < i1; ++k) {
          d[k] += alpha * p[k];
          const float rv = r[k] - alpha * ap[k];
          r[k] = rv;
          qb0 += rv * rv;
          qb1 += rv * (prec == COLAGB_PREC_JACOBI ? dinv[k] : 1.f) * rv;
        }
      }
    }
    float qb[2] = {qb0, qb1};
    cluster_sum_f<2, CL>(cl, qb, wpart, next_fslot());
    ++it;
    rn = sqrtf(qb[0]);
    float gamma_new = qb[1];
    bool restart = false;
    if (!(rn == rn)) {
      status = COLAGB_SYS_NAN;
      break;
    }
    if (rn <= delta * rmax || rn <= (float)a.tol || it >= a.max_inner ||
        (a.fallback && prec == COLAGB_PREC_FSAI && it - it_rep >= kJudgeSteps)) {
      // FP64 replacement: x += d, d = 0 ; r = b/|b| - A x
      it_rep = it;
      for (int64_t i = i0 + tid; i < i1; i += kCT) {
        X[i] += (double)d[i];
        d[i] = 0.f;
      }
      cl.sync();
      residual(q2);
      cluster_sum<2, CL>(cl, q2, next_slot(), red, bcast);
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
      gamma_new = (float)q2[1];
    }
    if (prec == COLAGB_PREC_FSAI || restart) {
      if (prec == COLAGB_PREC_FSAI) {
        fsai_t();
        cl.sync();
      }
      apply_z(q1);
      cluster_sum_f<1, CL>(cl, q1, wpart, next_fslot());
      gamma_new = q1[0];
    }
    const float beta = restart || gamma == 0.f ? 0.f : gamma_new / gamma;
    gamma = gamma_new;
    // C: p = z + beta p
    const bool zstored = prec == COLAGB_PREC_FSAI || restart;
    for (int64_t i = v0; i < i1; i += vstep) {
      if (i + 3 < i1) {
        float4 zv;
        if (zstored) {
          zv = *reinterpret_cast<const float4*>(z + i);
        } else {
          zv = *reinterpret_cast<const float4*>(r + i);
          if (prec == COLAGB_PREC_JACOBI) {
            const float4 di = *reinterpret_cast<const float4*>(dinv + i);
            zv.x *= di.x; zv.y *= di.y; zv.z *= di.z; zv.w *= di.w;
          }
        }
        const float4 pv = *reinterpret_cast<const float4*>(p + i);
        *reinterpret_cast<float4*>(p + i) =
            make_float4(zv.x + beta * pv.x, zv.y + beta * pv.y, zv.z + beta * pv.z, zv.w + beta * pv.w);
      } else {
        for (int64_t k = i; k < i1; ++k) {
          const float zv = zstored ? z[k] : (prec == COLAGB_PREC_JACOBI ? dinv[k] * r[k] : r[k]);
          p[k] = zv + beta * p[k];
        }
      }
    }
    cl.sync();
  }
  // finish: x += d, scale by |b|
  for (int64_t i = i0 + tid; i < i1; i += kCT) X[i] = (X[i] + (double)d[i]) * (bnorm > 0.0 ? bnorm : 1.0);
  if (rank == 0 && tid == 0) {
    int st = status == COLAGB_SYS_RUNNING ? COLAGB_SYS_MAX_ITERS : status;
    if (st == COLAGB_SYS_CONVERGED && a.prec_kind == COLAGB_PREC_FSAI && prec != COLAGB_PREC_FSAI)
      st = COLAGB_SYS_FALLBACK;
    if (a.out_status) a.out_status[s] = st;
    if (a.out_iters) a.out_iters[s] = it;
    if (a.out_relres) a.out_relres[s] = relres;
    if (a.out_nrep) a.out_nrep[s] = nrep;
  }
  cl.sync();  // no CTA leaves while another may still read its shared memory
}

template <int CL, bool BF>
static int launch_cluster(const ClusterArgs& a, cudaStream_t st) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(a.S * CL));
  cfg.blockDim = dim3(kCT);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = CL;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if (CL > 8)
    COLAGB_CUDA(cudaFuncSetAttribute(k_cluster_pcg<CL, BF>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
  int nclusters = 0;
  if (cudaOccupancyMaxActiveClusters(&nclusters, k_cluster_pcg<CL, BF>, &cfg) != cudaSuccess || nclusters < 1) {
    cudaGetLastError();
    return fail(COLAGB_ERR_UNSUPPORTED, "cluster PCG: cluster size not schedulable");
  }
  COLAGB_CUDA(cudaLaunchKernelEx(&cfg, k_cluster_pcg<CL, BF>, a));
  return COLAGB_OK;
}

// Called by colagb_cg_batched_csr_solve for the cluster schedule.
int cluster_pcg_solve(const colagb_batched_csr* A, const double* B, double* X, const colagb_ir_params* prm,
                      int32_t* iters, int32_t* status, double* relres, float* r, float* p, float* ap, float* d,
                      float* z, float* t, float* dinv, int* nrep, int cluster_size, __nv_bfloat16* v16,
                      float* dg16, cudaStream_t st) {
  ClusterArgs a;
  const bool bf = prm->matvec == COLAGB_MATVEC_BF16;
  a.v16 = v16;
  a.dg16 = dg16;
  a.dstride = A->shared_values ? 0 : A->n;
  if (bf) {
    const int64_t sets = A->shared_values ? 1 : A->num_systems;
    if (!v16 || !dg16) return fail(COLAGB_ERR_INVALID, "cluster PCG: BF16 matvec without its workspace");
    dim3 grid((unsigned)std::min<int64_t>(ceil_div(A->n, 256), (int64_t)num_sms() * 4), (unsigned)sets);
    k_bf16_consistent<<<grid, 256, 0, st>>>(A->indptr, A->indices, A->values, A->n, A->nnz, v16, dg16);
    COLAGB_CUDA(cudaGetLastError());
  }
  a.n = A->n;
  a.nnz = A->nnz;
  a.S = A->num_systems;
  a.vstride = A->shared_values ? 0 : A->nnz;
  a.indptr = A->indptr;
  a.indices = A->indices;
  a.vals = A->values;
  a.g_nnz = A->g_nnz;
  a.g_indptr = A->g_indptr;
  a.g_indices = A->g_indices;
  a.gt_indptr = A->gt_indptr;
  a.gt_indices = A->gt_indices;
  a.gt_perm = A->gt_perm;
  a.g_vals = A->g_values;
  a.B = B;
  a.X = X;
  a.r = r; a.p = p; a.ap = ap; a.d = d; a.z = z; a.t = t; a.dinv = dinv;
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
  if (bf) return cluster_size == 16 ? launch_cluster<16, true>(a, st) : launch_cluster<8, true>(a, st);
  return cluster_size == 16 ? launch_cluster<16, false>(a, st) : launch_cluster<8, false>(a, st);
}

}  // namespace colagb
