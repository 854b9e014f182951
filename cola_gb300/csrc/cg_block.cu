// Block schedule of the batched solver: many right-hand sides of ONE matrix advancing in lockstep.
//
// The reference's CG already runs a block of right-hand sides together: run_batched_cg keeps x, r, p
// as (n, k) arrays and per-column alpha / beta (cola/linalg/inverse/cg.py:94-154), so every step reads
// the matrix once for all k columns.  This kernel does the same on the GPU for a shared-values family
// (colagb_batched_csr.shared_values), with the batched solver's arithmetic: FP32 preconditioned CG
// (none / Jacobi), FP64 solution, FP64 residual replacement (reliable updates) and the FP64 true
// residual as the only convergence test, per column.
//
// Layout: the Krylov vectors are column-interleaved (n, kp) FP32 (kp = k padded to 4, 8, 16, 32, 64
// or 128), so one CSR entry multiplies a contiguous row of kp values of p: the kp / 4 threads of a row
// each take one 128-bit column quad.  The FP64 solution and the normalised right-hand side are
// (n, kp) FP64.  One persistent cooperative grid, rows split into contiguous ranges per CTA; per-column
// partial sums reduce in a fixed order (every CTA derives bit-identical scalars); three bounded grid
// barriers per step, two more per residual replacement.  A replacement happens for all columns at
// once, whenever one column's FP32 residual has dropped by inner_tol since the last one.
#include <algorithm>
#include <string>

#include "common.cuh"

namespace colagb {

constexpr int kBT = 256;        // threads per CTA
constexpr int kBMaxK = 128;     // columns per launch (the host splits wider blocks)

struct BlockArgs {
  int64_t n;
  int kp, q, S;                 // padded columns, column quads, real columns
  const int32_t* __restrict__ indptr;
  const int32_t* __restrict__ indices;
  const float* __restrict__ vals;
  const double* B;              // (S, n) right-hand sides
  double* X;                    // (S, n) solutions
  double* Bn;                   // (n, kp) B / |B|, per column
  double* X64;                  // (n, kp)
  float *R, *P, *AP, *D, *dinv; // (n, kp) x4, n
  float* pf;                    // [nb][3][kp]
  double* pd;                   // [nb][2][kp]
  int32_t* out_status;
  int32_t* out_iters;
  double* out_relres;
  int32_t* out_nrep;            // (1,) replacement count
  double tol, inner_tol;
  int max_inner, max_sweeps, jacobi;
  GridBarrier gb;
};

// Per-thread float4 partials of column quad (threadIdx % q, q a power of two <= 32) -> dst[0..4q) as
// one fixed-order sum: a shuffle tree over the lanes of a warp that share the quad, then warp by warp.
__device__ __forceinline__ void block_quad_partials(float4 v, int q, float* dst, float4* red) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int o = 16; o >= q; o >>= 1) {
    v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
    v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
    v.z += __shfl_xor_sync(0xffffffffu, v.z, o);
    v.w += __shfl_xor_sync(0xffffffffu, v.w, o);
  }
  if (lane < q) red[warp * 32 + lane] = v;  // lane l < q now holds the warp's sum for quad l
  __syncthreads();
  if ((int)threadIdx.x < q) {
    float4 t = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int w = 0; w < kBT / 32; ++w) {
      const float4 x = red[w * 32 + threadIdx.x];
      t.x += x.x; t.y += x.y; t.z += x.z; t.w += x.w;
    }
    reinterpret_cast<float4*>(dst)[threadIdx.x] = t;
  }
  __syncthreads();
}

// Column totals of FP32 partials over all CTAs, fixed order: into smem out[0..ncols).
__device__ __forceinline__ void grid_totals_f(const float* pf, int nb, int64_t stride, int ncols, float* out,
                                              float* tmp) {
  const int c = threadIdx.x & 31, g = threadIdx.x >> 5, ng = kBT / 32;
  for (int cb = 0; cb < ncols; cb += 32) {
    const int col = cb + c;
    float acc = 0.f;
    if (col < ncols)
      for (int b = g; b < nb; b += ng) acc += pf[(int64_t)b * stride + col];
    tmp[g * 32 + c] = acc;
    __syncthreads();
    if ((int)threadIdx.x < 32 && col < ncols) {
      float t = 0.f;
      for (int gg = 0; gg < ng; ++gg) t += tmp[gg * 32 + c];
      out[col] = t;
    }
    __syncthreads();
  }
}
__device__ __forceinline__ void grid_totals_d(const double* pd, int nb, int64_t stride, int ncols, double* out,
                                              double* tmp) {
  const int c = threadIdx.x & 31, g = threadIdx.x >> 5, ng = kBT / 32;
  for (int cb = 0; cb < ncols; cb += 32) {
    const int col = cb + c;
    double acc = 0.0;
    if (col < ncols)
      for (int b = g; b < nb; b += ng) acc += pd[(int64_t)b * stride + col];
    tmp[g * 32 + c] = acc;
    __syncthreads();
    if ((int)threadIdx.x < 32 && col < ncols) {
      double t = 0.0;
      for (int gg = 0; gg < ng; ++gg) t += tmp[gg * 32 + c];
      out[col] = t;
    }
    __syncthreads();
  }
}

// Four CTAs per SM (64 registers, no spills): the SpMM phase is latency-bound on index -> p-row
// gathers, and at two CTAs per SM (124 registers) only a quarter of the warp slots were occupied.
__global__ void __launch_bounds__(kBT, 4) k_block_ir(const BlockArgs a) {
  __shared__ float4 red[kBT];
  __shared__ double tmpd[kBT];
  __shared__ float tmpf[kBT];
  __shared__ float alpha[kBMaxK], beta[kBMaxK], gam[kBMaxK], gnew[kBMaxK], rn[kBMaxK], rmax[kBMaxK], pap[kBMaxK];
  __shared__ double bnorm[kBMaxK], relres[kBMaxK], tot64[2 * kBMaxK];
  __shared__ int frozen[kBMaxK], its[kBMaxK], status[kBMaxK];
  __shared__ int s_flag;

  const int64_t n = a.n;
  const int kp = a.kp, q = a.q;
  const int nb = gridDim.x;
  const int64_t rows = ceil_div(n, nb);
  const int64_t r0 = (int64_t)blockIdx.x * rows < n ? (int64_t)blockIdx.x * rows : n;
  const int64_t r1 = r0 + rows < n ? r0 + rows : n;
  const int64_t nu = (r1 - r0) * q;   // (row, quad) units of this CTA
  const int cq = (int)threadIdx.x % q;
  float* pf = a.pf + (int64_t)blockIdx.x * 3 * kp;
  double* pd = a.pd + (int64_t)blockIdx.x * 2 * kp;
  const float4* P4 = reinterpret_cast<const float4*>(a.P);
  float4* R4 = reinterpret_cast<float4*>(a.R);
  float4* Pw4 = reinterpret_cast<float4*>(a.P);
  float4* AP4 = reinterpret_cast<float4*>(a.AP);
  float4* D4 = reinterpret_cast<float4*>(a.D);

  // ---- setup: Bn = B (transposed), |B|^2 per column, X64 = D = 0, Jacobi diagonal ----
  for (int64_t u = threadIdx.x; u < (r1 - r0) * kp; u += kBT) {
    const int64_t i = r0 + u / kp;
    const int c = (int)(u % kp);
    a.Bn[i * kp + c] = c < a.S ? a.B[(int64_t)c * n + i] : 0.0;
    a.X64[i * kp + c] = 0.0;
    a.D[i * kp + c] = 0.f;
  }
  __syncthreads();
  if ((int)threadIdx.x < kp) {  // fixed-order per-column sum over this CTA's rows
    double acc = 0.0;
    for (int64_t i = r0; i < r1; ++i) {
      const double bv = a.Bn[i * kp + threadIdx.x];
      acc += bv * bv;
    }
    pd[threadIdx.x] = acc;
  }
  if (a.dinv)
    for (int64_t i = r0 + threadIdx.x; i < r1; i += kBT) {
      float dg = 0.f;
      for (int32_t j = a.indptr[i]; j < a.indptr[i + 1]; ++j)
        if (a.indices[j] == i) dg += a.vals[j];
      a.dinv[i] = dg != 0.f ? 1.f / dg : 1.f;
    }
  if (!grid_sync(a.gb)) return;
  grid_totals_d(a.pd, nb, 2 * kp, kp, tot64, tmpd);
  for (int c = threadIdx.x; c < kp; c += kBT) {
    const double bb = sqrt(tot64[c]);
    bnorm[c] = bb;
    its[c] = 0;
    frozen[c] = !(bb > 0.0);
    status[c] = bb > 0.0 ? COLAGB_SYS_RUNNING : (bb == 0.0 ? COLAGB_SYS_CONVERGED : COLAGB_SYS_NAN);
    relres[c] = bb > 0.0 ? 1.0 : 0.0;
  }
  __syncthreads();
  for (int64_t u = threadIdx.x; u < (r1 - r0) * kp; u += kBT) {
    const int c = (int)(u % kp);
    const int64_t e = (r0 + u / kp) * kp + c;
    a.Bn[e] = bnorm[c] > 0.0 ? a.Bn[e] / bnorm[c] : 0.0;
  }

  // FP64 residual replacement of every running column: X64 += D + alpha P (the step's correction,
  // which phase C would otherwise add to D), D = 0, R = Bn - A X64 (FP64), then |r64|^2 and <r, z>;
  // afterwards relres, gamma and rmax are set and converged columns frozen.
  auto replace = [&](bool first) -> bool {
    if (!first) {
      for (int64_t u = threadIdx.x; u < (r1 - r0) * kp; u += kBT) {
        const int64_t e = r0 * kp + u;
        const int c = (int)(u % kp);
        a.X64[e] += (double)(a.D[e] + alpha[c] * a.P[e]);
        a.D[e] = 0.f;
      }
      if (!grid_sync(a.gb)) return false;
    }
    double acc_rr = 0.0;
    float acc_rz = 0.f;
    const int col = (int)threadIdx.x % kp;  // kp divides kBT: thread t always takes column t % kp
    for (int64_t u = threadIdx.x; u < (r1 - r0) * kp; u += kBT) {
      const int64_t i = r0 + u / kp;
      double ax = 0.0;
      if (!first)
        for (int32_t j = a.indptr[i]; j < a.indptr[i + 1]; ++j)
          ax += (double)a.vals[j] * a.X64[(int64_t)a.indices[j] * kp + col];
      const double rv = frozen[col] ? 0.0 : a.Bn[i * kp + col] - ax;
      const float rf = (float)rv;
      a.R[i * kp + col] = rf;
      acc_rr += rv * rv;
      acc_rz += rf * (a.jacobi ? a.dinv[i] : 1.f) * rf;
    }
    // fixed-order per-column block sums (thread t accumulated column t % kp)
    tmpd[threadIdx.x] = acc_rr;
    tmpf[threadIdx.x] = acc_rz;
    __syncthreads();
    if ((int)threadIdx.x < kp) {
      double s1 = 0.0;
      float s2 = 0.f;
      for (int t = threadIdx.x; t < kBT; t += kp) {
        s1 += tmpd[t];
        s2 += tmpf[t];
      }
      pd[kp + threadIdx.x] = s1;
      pf[2 * kp + threadIdx.x] = s2;
    }
    __syncthreads();
    if (!grid_sync(a.gb)) return false;
    grid_totals_d(a.pd + kp, nb, 2 * kp, kp, tot64, tmpd);
    grid_totals_f(a.pf + 2 * kp, nb, 3 * kp, kp, gnew, tmpf);
    for (int c = threadIdx.x; c < kp; c += kBT) {
      if (frozen[c]) continue;
      const double rr = sqrt(tot64[c]);
      relres[c] = rr;
      rmax[c] = (float)rr;
      rn[c] = (float)rr;
      if (!(rr == rr)) {
        status[c] = COLAGB_SYS_NAN;
        frozen[c] = 1;
      } else if (rr <= a.tol) {
        status[c] = COLAGB_SYS_CONVERGED;
        frozen[c] = 1;
      }
    }
    __syncthreads();
    return true;
  };

  if (!replace(true)) return;
  for (int c = threadIdx.x; c < kp; c += kBT) gam[c] = gnew[c];
  __syncthreads();
  // p = z
  for (int64_t u = threadIdx.x; u < nu; u += kBT) {
    const int64_t i = r0 + u / q;
    const float4 r = R4[i * q + cq];
    const float d = a.jacobi ? a.dinv[i] : 1.f;
    Pw4[i * q + cq] = make_float4(d * r.x, d * r.y, d * r.z, d * r.w);
  }
  if (!grid_sync(a.gb)) return;

  int it = 0, nrep = 1;
  while (true) {
    if (threadIdx.x == 0) {
      int any = 0;
      for (int c = 0; c < kp; ++c) any |= !frozen[c];
      s_flag = any;
    }
    __syncthreads();
    if (!s_flag) break;
    // ---- A: AP = A P, <p, Ap> ----
    float4 part = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int64_t u = threadIdx.x; u < nu; u += kBT) {
      const int64_t i = r0 + u / q;
      const int32_t b = __ldg(a.indptr + i), e = __ldg(a.indptr + i + 1);
      float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
      // entries in groups of four: the group's indices and values, then its four p-row gathers, are
      // in flight together (one dependent index -> gather round trip per entry made this phase
      // latency-bound); the products are added in entry order as before
      for (int32_t j0 = b; j0 < e; j0 += 4) {
        int32_t col[4];
        float v[4];
#pragma unroll
        for (int t = 0; t < 4; ++t) {
          const bool ok = j0 + t < e;
          col[t] = ok ? __ldg(a.indices + j0 + t) : 0;
          v[t] = ok ? __ldg(a.vals + j0 + t) : 0.f;
        }
        float4 x[4];
#pragma unroll
        for (int t = 0; t < 4; ++t) x[t] = j0 + t < e ? P4[(int64_t)col[t] * q + cq] : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for (int t = 0; t < 4; ++t) {
          if (j0 + t < e) {
            acc.x += v[t] * x[t].x; acc.y += v[t] * x[t].y; acc.z += v[t] * x[t].z; acc.w += v[t] * x[t].w;
          }
        }
      }
      AP4[i * q + cq] = acc;
      const float4 p = P4[i * q + cq];
      part.x += p.x * acc.x; part.y += p.y * acc.y; part.z += p.z * acc.z; part.w += p.w * acc.w;
    }
    block_quad_partials(part, q, pf, red);
    if (!grid_sync(a.gb)) return;
    grid_totals_f(a.pf, nb, 3 * kp, kp, pap, tmpf);
    for (int c = threadIdx.x; c < kp; c += kBT) {
      if (frozen[c]) { alpha[c] = 0.f; continue; }
      if (!(pap[c] > 0.f)) {
        status[c] = pap[c] == pap[c] ? COLAGB_SYS_BREAKDOWN : COLAGB_SYS_NAN;
        frozen[c] = 1;
        alpha[c] = 0.f;
      } else {
        alpha[c] = gam[c] / pap[c];
      }
    }
    __syncthreads();
    // ---- B: r -= alpha Ap, |r|^2, <r, z> (d += alpha p waits for phase C, which reads p anyway) ----
    float4 prr = make_float4(0.f, 0.f, 0.f, 0.f), prz = make_float4(0.f, 0.f, 0.f, 0.f);
    const float4 al = make_float4(alpha[4 * cq], alpha[4 * cq + 1], alpha[4 * cq + 2], alpha[4 * cq + 3]);
    for (int64_t u = threadIdx.x; u < nu; u += kBT) {
      const int64_t i = r0 + u / q;
      const int64_t e = i * q + cq;
      const float4 ap = AP4[e];
      float4 r = R4[e];
      r.x -= al.x * ap.x; r.y -= al.y * ap.y; r.z -= al.z * ap.z; r.w -= al.w * ap.w;
      R4[e] = r;
      const float di = a.jacobi ? a.dinv[i] : 1.f;
      prr.x += r.x * r.x; prr.y += r.y * r.y; prr.z += r.z * r.z; prr.w += r.w * r.w;
      prz.x += r.x * di * r.x; prz.y += r.y * di * r.y; prz.z += r.z * di * r.z; prz.w += r.w * di * r.w;
    }
    block_quad_partials(prr, q, pf + kp, red);
    block_quad_partials(prz, q, pf + 2 * kp, red);
    if (!grid_sync(a.gb)) return;
    grid_totals_f(a.pf + kp, nb, 3 * kp, kp, rn, tmpf);
    grid_totals_f(a.pf + 2 * kp, nb, 3 * kp, kp, gnew, tmpf);
    ++it;
    if (threadIdx.x == 0) {
      int trig = 0;
      for (int c = 0; c < kp; ++c) {
        if (frozen[c]) continue;
        its[c] = it;
        const float r = sqrtf(rn[c]);
        rn[c] = r;
        if (!(r == r)) {
          status[c] = COLAGB_SYS_NAN;
          frozen[c] = 1;
          continue;
        }
        if (r <= (float)a.inner_tol * rmax[c] || r <= (float)a.tol) trig = 1;
      }
      if (it >= a.max_inner) trig = 1;
      s_flag = trig;
    }
    __syncthreads();
    const bool dpend = !s_flag;  // a replacement has already added this step's alpha p to x
    if (s_flag) {
      if (!replace(false)) return;
      ++nrep;
      if (it >= a.max_inner || nrep > a.max_sweeps) break;
    }
    // ---- C: beta, p = z + beta p ----
    for (int c = threadIdx.x; c < kp; c += kBT) {
      beta[c] = frozen[c] || gam[c] == 0.f ? 0.f : gnew[c] / gam[c];
      gam[c] = gnew[c];
    }
    __syncthreads();
    const float4 be = make_float4(beta[4 * cq], beta[4 * cq + 1], beta[4 * cq + 2], beta[4 * cq + 3]);
    for (int64_t u = threadIdx.x; u < nu; u += kBT) {
      const int64_t i = r0 + u / q;
      const int64_t e = i * q + cq;
      const float4 r = R4[e], p = P4[e];
      if (dpend) {
        float4 d = D4[e];
        d.x += al.x * p.x; d.y += al.y * p.y; d.z += al.z * p.z; d.w += al.w * p.w;
        D4[e] = d;
      }
      const float di = a.jacobi ? a.dinv[i] : 1.f;
      Pw4[e] = make_float4(di * r.x + be.x * p.x, di * r.y + be.y * p.y, di * r.z + be.z * p.z,
                           di * r.w + be.w * p.w);
    }
    if (!grid_sync(a.gb)) return;
  }
  // ---- finish: x = (X64 + D) |b| into the (S, n) output ----
  for (int64_t u = threadIdx.x; u < (r1 - r0) * kp; u += kBT) {
    const int64_t i = r0 + u / kp;
    const int c = (int)(u % kp);
    if (c < a.S) a.X[(int64_t)c * n + i] = (a.X64[i * kp + c] + (double)a.D[i * kp + c]) * bnorm[c];
  }
  if (blockIdx.x == 0) {
    for (int c = threadIdx.x; c < a.S; c += kBT) {
      int st = status[c] == COLAGB_SYS_RUNNING ? COLAGB_SYS_MAX_ITERS : status[c];
      if (a.out_status) a.out_status[c] = st;
      if (a.out_iters) a.out_iters[c] = its[c];
      if (a.out_relres) a.out_relres[c] = relres[c];
    }
    if (threadIdx.x == 0 && a.out_nrep) *a.out_nrep = nrep;
  }
}

int block_padded_width(int64_t k) {
  int kp = 4;
  while (kp < k) kp *= 2;
  return kp;
}

size_t block_workspace_bytes(int64_t n, int64_t S, int nb_max) {
  const int64_t k = S < kBMaxK ? S : kBMaxK;
  const int kp = block_padded_width(k);
  Bump ws = Bump::measuring();
  ws.take<double>((size_t)(n * kp));      // Bn
  ws.take<double>((size_t)(n * kp));      // X64
  for (int v = 0; v < 4; ++v) ws.take<float>((size_t)(n * kp));
  ws.take<float>((size_t)n);               // dinv
  ws.take<float>((size_t)nb_max * 3 * kp);
  ws.take<double>((size_t)nb_max * 2 * kp);
  ws.take<unsigned int>(8);
  ws.take<int>(4);
  return ws.peak;
}

int block_grid_blocks() {
  int occ = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_block_ir, kBT, 0) != cudaSuccess || occ < 1) {
    cudaGetLastError();
    return 0;
  }
  return num_sms() * (occ < 4 ? occ : 4);
}

// One shared-matrix block of up to kBMaxK right-hand sides (B, X: (S, n) FP64).
int block_pcg_solve(const colagb_batched_csr* A, const double* B, double* X, const colagb_ir_params* prm,
                    int32_t* iters, int32_t* status, double* relres, void* ws_ptr, size_t ws_bytes, int* max_rep,
                    cudaStream_t st) {
  const int64_t n = A->n;
  for (int64_t s0 = 0; s0 < A->num_systems; s0 += kBMaxK) {
    const int S = (int)std::min<int64_t>(kBMaxK, A->num_systems - s0);
    const int kp = block_padded_width(S);
    const int nb = block_grid_blocks();
    if (nb < 1) return fail(COLAGB_ERR_UNSUPPORTED, "block schedule: kernel cannot be resident");
    Bump ws(ws_ptr, ws_bytes);
    BlockArgs a;
    a.n = n;
    a.kp = kp;
    a.q = kp / 4;
    a.S = S;
    a.indptr = A->indptr;
    a.indices = A->indices;
    a.vals = A->values;
    a.B = B + s0 * n;
    a.X = X + s0 * n;
    a.Bn = ws.take<double>((size_t)(n * kp));
    a.X64 = ws.take<double>((size_t)(n * kp));
    a.R = ws.take<float>((size_t)(n * kp));
    a.P = ws.take<float>((size_t)(n * kp));
    a.AP = ws.take<float>((size_t)(n * kp));
    a.D = ws.take<float>((size_t)(n * kp));
    float* dinv = ws.take<float>((size_t)n);
    a.pf = ws.take<float>((size_t)nb * 3 * kp);
    a.pd = ws.take<double>((size_t)nb * 2 * kp);
    unsigned int* bar = ws.take<unsigned int>(8);
    int* nrep = ws.take<int>(4);
    if (ws.overflow()) return fail(COLAGB_ERR_WORKSPACE, "block schedule: workspace too small");
    a.jacobi = prm->preconditioner == COLAGB_PREC_JACOBI ? 1 : 0;
    a.dinv = a.jacobi ? dinv : nullptr;
    a.out_status = status ? status + s0 : nullptr;
    a.out_iters = iters ? iters + s0 : nullptr;
    a.out_relres = relres ? relres + s0 : nullptr;
    a.out_nrep = nrep;
    a.tol = prm->tol;
    a.inner_tol = prm->inner_tol;
    a.max_inner = prm->max_inner_iters;
    a.max_sweeps = prm->max_sweeps;
    a.gb.count = bar;
    a.gb.generation = bar + 1;
    a.gb.err = reinterpret_cast<int*>(bar + 2);
    a.gb.nblocks = (unsigned)nb;
    a.gb.spin_limit = prm->spin_limit > 0 ? prm->spin_limit : kDefaultSpinLimit;
    COLAGB_CUDA(cudaMemsetAsync(bar, 0, 8 * sizeof(unsigned int), st));
    void* args[] = {&a};
    COLAGB_CUDA(cudaLaunchCooperativeKernel((const void*)k_block_ir, dim3(nb), dim3(kBT), args, 0, st));
    int h[2] = {0, 0};
    COLAGB_CUDA(cudaMemcpyAsync(&h[0], bar + 2, sizeof(int), cudaMemcpyDeviceToHost, st));
    COLAGB_CUDA(cudaMemcpyAsync(&h[1], nrep, sizeof(int), cudaMemcpyDeviceToHost, st));
    COLAGB_CUDA(cudaStreamSynchronize(st));
    if (h[0] != 0) return fail(COLAGB_ERR_TIMEOUT, "block schedule: a grid barrier timed out");
    if (h[1] > *max_rep) *max_rep = h[1];
  }
  return COLAGB_OK;
}

}  // namespace colagb
