// Learned factored sparse approximate inverse (FSAI) preconditioner for 5-point operators on an
// m x m grid: a small convolutional network reads the operator's coefficients and outputs the
// lower-triangular factor G on A's own lower pattern {N = p-m, W = p-1, C = p}; P = G^T G.
//
// Parametrisation: with d = diag(A), a_N = A[p, p-m], a_W = A[p, p-1] and the Schur complement
// s_p = d_p - a_N^2 / d_N - a_W^2 / d_W, the closed-form FSAI row of this pattern is
//   G_C = 1/sqrt(s_p),  G_N = -(a_N/d_N)/sqrt(s_p),  G_W = -(a_W/d_W)/sqrt(s_p).
// The network's outputs (o1, o2) per cell reshape it, H = (G_N (1 + o1), G_W (1 + o2), G_C), and each
// row is renormalised so that (G A G^T)_pp = 1 (the FSAI normalisation; the closed form already
// satisfies it, so o = 0 reproduces closed-form FSAI).  G_C > 0 for any o, so P is SPD whatever the
// network predicts, and diag(G A G^T) = 1 keeps its largest eigenvalue bounded.
//
// Training loss per system (pairs (r, e) with A e = r, e from this project's CG):
//   l = ||P r - e||_A^2 / ||e||_A^2 = (v^T A v - 2 v^T r + e^T r) / (e^T r),  v = G^T G r.
// Its gradient: dl/dv = 2 (A v - r) / (e^T r) =: g;  dl/dG_pq = t_p g_q + (G g)_p r_q with t = G r.
//
// Layouts: grid fields are (S, C, m, m) float32, row-major cells p = i*m + j.
#include <cmath>
#include <string>

#include "common.cuh"

namespace colagb {

// ---------------------------------------------------------------------------------------------
// stencil extraction: CSR values (S, nnz) on the grid's 5-point pattern -> (S, 5, m, m) [N, W, C, E, S]
__global__ void k_grid5_stencil(const int32_t* __restrict__ indptr, const int32_t* __restrict__ indices,
                                const float* __restrict__ values, int64_t nnz, int64_t m, int64_t S,
                                float* __restrict__ st, int* err) {
  const int64_t n = m * m;
  for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < S * n; u += (int64_t)gridDim.x * blockDim.x) {
    const int64_t s = u / n, p = u % n;
    float o[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
    for (int32_t e = indptr[p]; e < indptr[p + 1]; ++e) {
      const int64_t c = indices[e];
      const float v = values[s * nnz + e];
      const int64_t d = c - p;
      if (d == -m) o[0] += v;
      else if (d == -1) o[1] += v;
      else if (d == 0) o[2] += v;
      else if (d == 1) o[3] += v;
      else if (d == m) o[4] += v;
      else atomicExch(err, 1);
    }
    float* base = st + s * 5 * n + p;
#pragma unroll
    for (int k = 0; k < 5; ++k) base[k * n] = o[k];
  }
}

__device__ __forceinline__ float at5(const float* st, int64_t n, int k, int64_t p) { return st[k * n + p]; }

// features (S, 6, m, m): -a_N/d, -a_W/d, -a_E/d, -a_S/d, log(d/d_N), log(d/d_W)  (0 where absent)
__global__ void k_fsai_features(const float* __restrict__ st, int64_t m, int64_t S, float* __restrict__ f) {
  const int64_t n = m * m;
  for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < S * n; u += (int64_t)gridDim.x * blockDim.x) {
    const int64_t s = u / n, p = u % n;
    const int64_t i = p / m, j = p % m;
    const float* a = st + s * 5 * n;
    const float d = at5(a, n, 2, p);
    float* o = f + s * 6 * n + p;
    o[0] = -at5(a, n, 0, p) / d;
    o[1 * n] = -at5(a, n, 1, p) / d;
    o[2 * n] = -at5(a, n, 3, p) / d;
    o[3 * n] = -at5(a, n, 4, p) / d;
    o[4 * n] = i > 0 ? logf(d / at5(a, n, 2, p - m)) : 0.f;
    o[5 * n] = j > 0 ? logf(d / at5(a, n, 2, p - 1)) : 0.f;
  }
}

// closed-form FSAI coefficients (S, 3, m, m): [N, W, C] rows of G for o = 0
__device__ __forceinline__ void fsai_closed_form(const float* a, int64_t n, int64_t m, int64_t p, float& fN, float& fW,
                                                 float& fC) {
  const int64_t i = p / m, j = p % m;
  const float d = at5(a, n, 2, p);
  float sch = d, cN = 0.f, cW = 0.f;
  if (i > 0) {
    const float aN = at5(a, n, 0, p), dN = at5(a, n, 2, p - m);
    sch -= aN * aN / dN;
    cN = -aN / dN;
  }
  if (j > 0) {
    const float aW = at5(a, n, 1, p), dW = at5(a, n, 2, p - 1);
    sch -= aW * aW / dW;
    cW = -aW / dW;
  }
  const float is = rsqrtf(sch);
  fC = is;
  fN = cN * is;
  fW = cW * is;
}

// One row of G from the network output (o1, o2): H = (fN (1 + tanh o1), fW (1 + tanh o2), fC) -- each
// off-diagonal between 0 and twice its closed-form value -- then the FSAI
// normalisation G = H / sqrt(s), s = (H A H^T)_pp, so that diag(G A G^T) = 1 whatever the network
// predicts (the largest eigenvalue of G A G^T stays bounded; only the shape of each row is learned).
// For o = 0, H is the closed-form row and s = 1.  Also returns the pieces the gradient needs.
struct FsaiRow {
  float fN, fW, fC;  // closed form
  float hN, hW, hC;  // before normalisation
  float d, dN, dW, aN, aW;
  float s;
};
__device__ __forceinline__ FsaiRow fsai_row(const float* a, int64_t n, int64_t m, int64_t p, float o1, float o2) {
  FsaiRow r;
  fsai_closed_form(a, n, m, p, r.fN, r.fW, r.fC);
  const int64_t i = p / m, j = p % m;
  r.d = at5(a, n, 2, p);
  r.dN = i > 0 ? at5(a, n, 2, p - m) : 0.f;
  r.dW = j > 0 ? at5(a, n, 2, p - 1) : 0.f;
  r.aN = i > 0 ? at5(a, n, 0, p) : 0.f;
  r.aW = j > 0 ? at5(a, n, 1, p) : 0.f;
  r.hN = r.fN * (1.f + tanhf(o1));
  r.hW = r.fW * (1.f + tanhf(o2));
  r.hC = r.fC;
  r.s = r.hC * r.hC * r.d + r.hN * r.hN * r.dN + r.hW * r.hW * r.dW + 2.f * r.hC * (r.hN * r.aN + r.hW * r.aW);
  return r;
}

// G stencil (S, 3, m, m) [N, W, C] from the network output o (S, 3, m, m) (o may be null: o = 0);
// channel 0 of o is not used (the normalisation fixes each row's scale).
__global__ void k_fsai_assemble(const float* __restrict__ st, const float* __restrict__ o, int64_t m, int64_t S,
                                float* __restrict__ g) {
  const int64_t n = m * m;
  for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < S * n; u += (int64_t)gridDim.x * blockDim.x) {
    const int64_t s = u / n, p = u % n;
    const float o1 = o ? o[s * 3 * n + n + p] : 0.f, o2 = o ? o[s * 3 * n + 2 * n + p] : 0.f;
    const FsaiRow r = fsai_row(st + s * 5 * n, n, m, p, o1, o2);
    const float is = o ? rsqrtf(r.s) : 1.f;
    g[s * 3 * n + p] = r.hN * is;
    g[s * 3 * n + n + p] = r.hW * is;
    g[s * 3 * n + 2 * n + p] = r.hC * is;
  }
}

// G stencil -> compact CSR values (S, g_nnz) in the lower pattern's order [N, W, C] (absent skipped)
__global__ void k_fsai_compact(const float* __restrict__ g, const int32_t* __restrict__ g_indptr, int64_t m, int64_t S,
                               int64_t g_nnz, float* __restrict__ out) {
  const int64_t n = m * m;
  for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < S * n; u += (int64_t)gridDim.x * blockDim.x) {
    const int64_t s = u / n, p = u % n;
    const int64_t i = p / m, j = p % m;
    int64_t e = g_indptr[p];
    float* o = out + s * g_nnz;
    if (i > 0) o[e++] = g[s * 3 * n + p];
    if (j > 0) o[e++] = g[s * 3 * n + n + p];
    o[e] = g[s * 3 * n + 2 * n + p];
  }
}

// ---------------------------------------------------------------------------------------------
// 3x3 convolution, zero padding 1, stride 1.  in (B, CIN, H, W), w (COUT, CIN, 3, 3), b (COUT).
template <int COUT>
__global__ void __launch_bounds__(256) k_conv3_fwd(const float* __restrict__ in, int cin, int H, int W,
                                                   const float* __restrict__ w, const float* __restrict__ bias,
                                                   int relu, float* __restrict__ out) {
  extern __shared__ float sw[];  // COUT * cin * 9 weights
  __shared__ float tile[18][18];
  const int bimg = blockIdx.z;
  const int x0 = blockIdx.x * 16, y0 = blockIdx.y * 16;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  for (int q = threadIdx.x; q < COUT * cin * 9; q += 256) sw[q] = w[q];
  float acc[COUT];
#pragma unroll
  for (int c = 0; c < COUT; ++c) acc[c] = bias ? bias[c] : 0.f;
  const int64_t plane = (int64_t)H * W;
  for (int ci = 0; ci < cin; ++ci) {
    const float* src = in + ((int64_t)bimg * cin + ci) * plane;
    __syncthreads();
    for (int q = threadIdx.x; q < 18 * 18; q += 256) {
      const int yy = y0 - 1 + q / 18, xx = x0 - 1 + q % 18;
      tile[q / 18][q % 18] = (yy >= 0 && yy < H && xx >= 0 && xx < W) ? src[(int64_t)yy * W + xx] : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int ky = 0; ky < 3; ++ky)
#pragma unroll
      for (int kx = 0; kx < 3; ++kx) {
        const float v = tile[ty + ky][tx + kx];
#pragma unroll
        for (int c = 0; c < COUT; ++c) acc[c] += sw[(c * cin + ci) * 9 + ky * 3 + kx] * v;
      }
  }
  const int y = y0 + ty, x = x0 + tx;
  if (y < H && x < W) {
#pragma unroll
    for (int c = 0; c < COUT; ++c) {
      const float v = acc[c];
      out[((int64_t)bimg * COUT + c) * plane + (int64_t)y * W + x] = relu ? fmaxf(v, 0.f) : v;
    }
  }
}

// ---------------------------------------------------------------------------------------------
// The preconditioner build of the trained network in one pass.  One CTA builds a 32 x 32 tile of
// cells: features -> conv 6->16 (ReLU) -> conv 16->16 (ReLU) -> conv 16->3, of whose output only
// channels 1 and 2 are evaluated (the assembly reads no other) -> normalised G row -> CSR values.
// Each layer is evaluated on the tile plus the halo the layers after it read (38^2 feature cells,
// then 36^2, 34^2, 32^2), all in shared memory.  Cells outside the grid hold 0 in every layer -- the
// zero padding of the layer-by-layer evaluation -- and every output is the same chain of FMAs in
// the same order as in k_fsai_features -> k_conv3_fwd x 3 -> k_fsai_assemble -> k_fsai_compact.
//
// Work split: item k of thread t covers cell lt + k * (512 / NG) of the layer's region and output
// channels grp * CG .. grp * CG + CG - 1 (grp = t / (512 / NG)), so that the CG weights of one
// (input channel, tap) -- one or two 128-bit shared loads, the same address for the whole warp --
// serve every item of the thread.  Layer 1: 1296 cells x 16 channels as 3 items; layer 2: 1156
// cells as 5 items of 8 channels; layer 3: 1024 cells x 2 channels as 2 items.
constexpr int kNetTile = 32;
constexpr int kNetThreads = 512;
constexpr int kNetF = kNetTile + 6;               // side of the feature region
constexpr int kNetBufA = 16 * (kNetTile + 2) * (kNetTile + 2);  // features (6 x 38^2), later h2 (16 x 34^2)
constexpr int kNetBufB = 16 * (kNetTile + 4) * (kNetTile + 4);  // h1 (16 x 36^2)
constexpr int kNetW1 = 6 * 9 * 16, kNetW2 = 16 * 9 * 16, kNetW3 = 16 * 9 * 2;
constexpr int kNetParams = 16 * 6 * 9 + 16 + 16 * 16 * 9 + 16 + 3 * 16 * 9 + 3;  // FsaiNet's flat layout
constexpr size_t kNetSmemBytes = (size_t)(kNetBufA + kNetBufB + kNetW1 + kNetW2 + kNetW3 + 16 + 16 + 4) * sizeof(float);
static_assert(6 * kNetF * kNetF <= kNetBufA, "features fit in buffer A");
static_assert(kNetBufA % 4 == 0 && kNetBufB % 4 == 0 && kNetW1 % 4 == 0, "weights 16-byte aligned");

template <int CIN, int COUT, int NG, int RIN, int PPT>
__device__ __forceinline__ void net_conv(const float* in, const float* w, const float* b,
                                         float (&acc)[PPT][COUT / NG], int& grp, int& lt) {
  constexpr int CG = COUT / NG, TPG = kNetThreads / NG, ROUT = RIN - 2, NP = ROUT * ROUT, PIN = RIN * RIN;
  static_assert(PPT * TPG >= NP && (PPT - 1) * TPG < NP, "items per thread");
  static_assert(CG % 4 == 0 || CG == 2, "weight vector width");
  grp = threadIdx.x / TPG;
  lt = threadIdx.x % TPG;
  int base[PPT];
#pragma unroll
  for (int k = 0; k < PPT; ++k) {
    const int q = lt + k * TPG;
    base[k] = q < NP ? (q / ROUT) * RIN + q % ROUT : 0;  // items past the region read cell 0, discarded
  }
  const float* wg = w + grp * CG;
#pragma unroll
  for (int k = 0; k < PPT; ++k)
#pragma unroll
    for (int c = 0; c < CG; ++c) acc[k][c] = b[grp * CG + c];
#pragma unroll 1
  for (int ci = 0; ci < CIN; ++ci) {
    const float* src = in + ci * PIN;
    const float* wc = wg + ci * 9 * COUT;
#pragma unroll
    for (int t = 0; t < 9; ++t) {
      const int off = (t / 3) * RIN + t % 3;
      float wv[CG];
      if constexpr (CG % 4 == 0) {
#pragma unroll
        for (int c4 = 0; c4 < CG / 4; ++c4) {
          const float4 x = *reinterpret_cast<const float4*>(wc + t * COUT + 4 * c4);
          wv[4 * c4] = x.x; wv[4 * c4 + 1] = x.y; wv[4 * c4 + 2] = x.z; wv[4 * c4 + 3] = x.w;
        }
      } else {
        const float2 x = *reinterpret_cast<const float2*>(wc + t * COUT);
        wv[0] = x.x; wv[1] = x.y;
      }
#pragma unroll
      for (int k = 0; k < PPT; ++k) {
        const float v = src[base[k] + off];
#pragma unroll
        for (int c = 0; c < CG; ++c) acc[k][c] += wv[c] * v;
      }
    }
  }
}

// ReLU'd layer output into its shared region (ROUT^2 cells from grid cell (oy, ox)); 0 off the grid
template <int COUT, int NG, int ROUT, int PPT>
__device__ __forceinline__ void net_store(const float (&acc)[PPT][COUT / NG], int grp, int lt, float* out, int oy, int ox,
                                          int64_t m) {
  constexpr int CG = COUT / NG, TPG = kNetThreads / NG, NP = ROUT * ROUT;
#pragma unroll
  for (int k = 0; k < PPT; ++k) {
    const int q = lt + k * TPG;
    if (q < NP) {
      const int y = oy + q / ROUT, x = ox + q % ROUT;
      const bool inside = y >= 0 && y < m && x >= 0 && x < m;
#pragma unroll
      for (int c = 0; c < CG; ++c) out[(grp * CG + c) * NP + q] = inside ? fmaxf(acc[k][c], 0.f) : 0.f;
    }
  }
}

__global__ void __launch_bounds__(kNetThreads, 1)
    k_fsai_net_build(const float* __restrict__ st, const float* __restrict__ params, int64_t m, int64_t S,
                     const int32_t* __restrict__ g_indptr, int64_t g_nnz, float* __restrict__ out,
                     unsigned int* tile_counter) {
  extern __shared__ __align__(16) float nsm[];
  float* bufA = nsm;
  float* bufB = bufA + kNetBufA;
  float* w1 = bufB + kNetBufB;
  float* w2 = w1 + kNetW1;
  float* w3 = w2 + kNetW2;
  float* b1 = w3 + kNetW3;
  float* b2 = b1 + 16;
  float* b3 = b2 + 16;
  const int tid = threadIdx.x;
  // weights W (cout, cin, 3, 3) then b (cout) per layer -> [(ci * 9 + tap) * cout + co]
  for (int u = tid; u < 16 * 6 * 9; u += kNetThreads) w1[((u / 9) % 6 * 9 + u % 9) * 16 + u / 54] = params[u];
  for (int u = tid; u < 16 * 16 * 9; u += kNetThreads) w2[((u / 9) % 16 * 9 + u % 9) * 16 + u / 144] = params[880 + u];
  for (int u = tid; u < 2 * 16 * 9; u += kNetThreads) {
    const int co = 1 + u / 144;  // output channels 1 and 2 of the last layer
    w3[((u / 9) % 16 * 9 + u % 9) * 2 + co - 1] = params[3200 + co * 144 + u % 144];
  }
  if (tid < 16) {
    b1[tid] = params[864 + tid];
    b2[tid] = params[3184 + tid];
  }
  if (tid < 2) b3[tid] = params[3632 + 1 + tid];

  const int64_t n = m * m;
  const int64_t side = (m + kNetTile - 1) / kNetTile, per_sys = side * side;
  __shared__ unsigned int s_tile;
  // tiles from an atomic counter, so that the CTAs that get an SM early (e.g. beside another
  // kernel that holds the others) take the work of the ones that start late
  for (int64_t tile0 = blockIdx.x;; tile0 += gridDim.x) {
    __syncthreads();  // weights in; the previous tile's reads of buffer A and of s_tile done
    if (tile_counter) {
      if (tid == 0) s_tile = atomicAdd(tile_counter, 1u);
      __syncthreads();
    }
    const int64_t tile = tile_counter ? (int64_t)s_tile : tile0;
    if (tile >= per_sys * S) break;
    const int64_t s = tile / per_sys, r = tile % per_sys;
    const int y0 = (int)(r / side) * kNetTile, x0 = (int)(r % side) * kNetTile;
    const float* a = st + s * 5 * n;
    // features (as k_fsai_features) on the 38^2 region from (y0 - 3, x0 - 3)
    for (int q = tid; q < kNetF * kNetF; q += kNetThreads) {
      const int y = y0 - 3 + q / kNetF, x = x0 - 3 + q % kNetF;
      float f[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
      if (y >= 0 && y < m && x >= 0 && x < m) {
        const int64_t p = (int64_t)y * m + x;
        const float d = at5(a, n, 2, p);
        f[0] = -at5(a, n, 0, p) / d;
        f[1] = -at5(a, n, 1, p) / d;
        f[2] = -at5(a, n, 3, p) / d;
        f[3] = -at5(a, n, 4, p) / d;
        f[4] = y > 0 ? logf(d / at5(a, n, 2, p - m)) : 0.f;
        f[5] = x > 0 ? logf(d / at5(a, n, 2, p - 1)) : 0.f;
      }
#pragma unroll
      for (int c = 0; c < 6; ++c) bufA[c * kNetF * kNetF + q] = f[c];
    }
    __syncthreads();
    {
      float acc[3][16];
      int grp, lt;
      net_conv<6, 16, 1, kNetTile + 6, 3>(bufA, w1, b1, acc, grp, lt);
      net_store<16, 1, kNetTile + 4, 3>(acc, grp, lt, bufB, y0 - 2, x0 - 2, m);
    }
    __syncthreads();
    {
      float acc[5][8];
      int grp, lt;
      net_conv<16, 16, 2, kNetTile + 4, 5>(bufB, w2, b2, acc, grp, lt);
      net_store<16, 2, kNetTile + 2, 5>(acc, grp, lt, bufA, y0 - 1, x0 - 1, m);
    }
    __syncthreads();
    {
      float acc[2][2];
      int grp, lt;
      net_conv<16, 2, 1, kNetTile + 2, 2>(bufA, w3, b3, acc, grp, lt);
      float* o = out + s * g_nnz;
#pragma unroll
      for (int k = 0; k < 2; ++k) {
        const int q = lt + k * kNetThreads;
        const int y = y0 + q / kNetTile, x = x0 + q % kNetTile;
        if (y < m && x < m) {
          const int64_t p = (int64_t)y * m + x;
          const FsaiRow row = fsai_row(a, n, m, p, acc[k][0], acc[k][1]);
          const float is = rsqrtf(row.s);
          int64_t e = g_indptr[p];
          if (y > 0) o[e++] = row.hN * is;
          if (x > 0) o[e++] = row.hW * is;
          o[e] = row.hC * is;
        }
      }
    }
  }
}

// closed-form FSAI straight to CSR values (k_fsai_assemble with o = 0, then k_fsai_compact)
__global__ void k_fsai_closed_build(const float* __restrict__ st, int64_t m, int64_t S,
                                    const int32_t* __restrict__ g_indptr, int64_t g_nnz, float* __restrict__ out) {
  const int64_t n = m * m;
  for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < S * n; u += (int64_t)gridDim.x * blockDim.x) {
    const int64_t s = u / n, p = u % n;
    const int64_t i = p / m, j = p % m;
    float fN, fW, fC;
    fsai_closed_form(st + s * 5 * n, n, m, p, fN, fW, fC);
    float* o = out + s * g_nnz;
    int64_t e = g_indptr[p];
    if (i > 0) o[e++] = fN;
    if (j > 0) o[e++] = fW;
    o[e] = fC;
  }
}

// grad_in (B, CIN, H, W) from grad_out (B, cout, H, W); when `act` is given the forward output
// was ReLU(act) and grad_out is masked by act > 0.
template <int CIN>
__global__ void __launch_bounds__(256) k_conv3_bwd_data(const float* __restrict__ gout, const float* __restrict__ act,
                                                        int cout, int H, int W, const float* __restrict__ w,
                                                        float* __restrict__ gin) {
  extern __shared__ float sw[];  // cout * CIN * 9
  __shared__ float tile[18][18];
  const int bimg = blockIdx.z;
  const int x0 = blockIdx.x * 16, y0 = blockIdx.y * 16;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  for (int q = threadIdx.x; q < cout * CIN * 9; q += 256) sw[q] = w[q];
  float acc[CIN];
#pragma unroll
  for (int c = 0; c < CIN; ++c) acc[c] = 0.f;
  const int64_t plane = (int64_t)H * W;
  for (int co = 0; co < cout; ++co) {
    const float* g = gout + ((int64_t)bimg * cout + co) * plane;
    const float* a = act ? act + ((int64_t)bimg * cout + co) * plane : nullptr;
    __syncthreads();
    for (int q = threadIdx.x; q < 18 * 18; q += 256) {
      const int yy = y0 - 1 + q / 18, xx = x0 - 1 + q % 18;
      float v = 0.f;
      if (yy >= 0 && yy < H && xx >= 0 && xx < W) {
        const int64_t o = (int64_t)yy * W + xx;
        v = g[o];
        if (a && !(a[o] > 0.f)) v = 0.f;
      }
      tile[q / 18][q % 18] = v;
    }
    __syncthreads();
#pragma unroll
    for (int ky = 0; ky < 3; ++ky)
#pragma unroll
      for (int kx = 0; kx < 3; ++kx) {
        const float v = tile[ty + 2 - ky][tx + 2 - kx];
#pragma unroll
        for (int c = 0; c < CIN; ++c) acc[c] += sw[(co * CIN + c) * 9 + ky * 3 + kx] * v;
      }
  }
  const int y = y0 + ty, x = x0 + tx;
  if (y < H && x < W) {
#pragma unroll
    for (int c = 0; c < CIN; ++c) gin[((int64_t)bimg * CIN + c) * plane + (int64_t)y * W + x] = acc[c];
  }
}

// grad_w partials: part[blk][(co*cin + ci)*9 + k] and part_b[blk][co]; blocks stride over tiles.
__global__ void __launch_bounds__(256) k_conv3_bwd_weight(const float* __restrict__ gout, const float* __restrict__ act,
                                                          const float* __restrict__ in, int B, int cin, int cout,
                                                          int H, int W, float* __restrict__ part) {
  extern __shared__ float sm[];
  float* gt = sm;                         // cout * 256 (masked grad_out tile)
  float* it = sm + cout * 256;            // cin * 324 (input tile with halo)
  const int nw = cout * cin * 9;
  const int tiles_x = (W + 15) / 16, tiles_y = (H + 15) / 16;
  const int ntiles = tiles_x * tiles_y * B;
  const int64_t plane = (int64_t)H * W;
  float accw[12];  // up to 12 entries per thread (nw <= 3072)
  float accb = 0.f;
#pragma unroll
  for (int q = 0; q < 12; ++q) accw[q] = 0.f;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int bimg = tile / (tiles_x * tiles_y);
    const int rem = tile % (tiles_x * tiles_y);
    const int y0 = (rem / tiles_x) * 16, x0 = (rem % tiles_x) * 16;
    __syncthreads();
    for (int q = threadIdx.x; q < cout * 256; q += 256) {
      const int co = q / 256, yy = y0 + (q % 256) / 16, xx = x0 + (q % 16);
      float v = 0.f;
      if (yy < H && xx < W) {
        const int64_t o = ((int64_t)bimg * cout + co) * plane + (int64_t)yy * W + xx;
        v = gout[o];
        if (act && !(act[o] > 0.f)) v = 0.f;
      }
      gt[q] = v;
    }
    for (int q = threadIdx.x; q < cin * 324; q += 256) {
      const int ci = q / 324, yy = y0 - 1 + (q % 324) / 18, xx = x0 - 1 + (q % 18);
      it[q] = (yy >= 0 && yy < H && xx >= 0 && xx < W) ? in[((int64_t)bimg * cin + ci) * plane + (int64_t)yy * W + xx]
                                                       : 0.f;
    }
    __syncthreads();
    for (int q = 0; q < 12; ++q) {
      const int e = threadIdx.x + q * 256;
      if (e >= nw) break;
      const int co = e / (cin * 9), ci = (e / 9) % cin, k = e % 9, ky = k / 3, kx = k % 3;
      const float* g = gt + co * 256;
      const float* x = it + ci * 324;
      float s = 0.f;
      for (int py = 0; py < 16; ++py)
#pragma unroll 4
        for (int px = 0; px < 16; ++px) s += g[py * 16 + px] * x[(py + ky) * 18 + px + kx];
      accw[q] += s;
    }
    if (threadIdx.x < cout) {
      const float* g = gt + threadIdx.x * 256;
      float s = 0.f;
      for (int q = 0; q < 256; ++q) s += g[q];
      accb += s;
    }
  }
  float* out = part + (int64_t)blockIdx.x * (nw + cout);
  for (int q = 0; q < 12; ++q) {
    const int e = threadIdx.x + q * 256;
    if (e < nw) out[e] = accw[q];
  }
  if (threadIdx.x < cout) out[nw + threadIdx.x] = accb;
}

__global__ void k_sum_partials(const float* __restrict__ part, int nblk, int len, float* __restrict__ out, int accumulate) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < len; e += gridDim.x * blockDim.x) {
    float s = 0.f;
    for (int b = 0; b < nblk; ++b) s += part[(int64_t)b * len + e];
    out[e] = accumulate ? out[e] + s : s;
  }
}

// ---------------------------------------------------------------------------------------------
// loss and gradient.  gs: G stencil (S, 3, m, m) [N, W, C]; st: A stencil (S, 5, m, m);
// r, e: (S, n) pairs; sc: per-system FP64 scalars [3][S] = e^T r, v^T w, v^T r.
__device__ __forceinline__ float g_row(const float* gs, int64_t n, int64_t m, int64_t p, const float* x) {
  const int64_t i = p / m, j = p % m;
  float v = gs[2 * n + p] * x[p];
  if (i > 0) v += gs[p] * x[p - m];
  if (j > 0) v += gs[n + p] * x[p - 1];
  return v;
}
__device__ __forceinline__ float gt_row(const float* gs, int64_t n, int64_t m, int64_t q, const float* x) {
  const int64_t i = q / m, j = q % m;
  float v = gs[2 * n + q] * x[q];
  if (i < m - 1) v += gs[q + m] * x[q + m];
  if (j < m - 1) v += gs[n + q + 1] * x[q + 1];
  return v;
}
__device__ __forceinline__ float a_row(const float* st, int64_t n, int64_t m, int64_t p, const float* x) {
  const int64_t i = p / m, j = p % m;
  float v = st[2 * n + p] * x[p];
  if (i > 0) v += st[p] * x[p - m];
  if (j > 0) v += st[n + p] * x[p - 1];
  if (j < m - 1) v += st[3 * n + p] * x[p + 1];
  if (i < m - 1) v += st[4 * n + p] * x[p + m];
  return v;
}

// d(loss)/d(o) of one row from d(loss)/d(G_C, G_N, G_W) at row p.  G = H / sqrt(s(H)),
// H = (fN (1 + tanh o1), fW (1 + tanh o2), fC):
//   dl/dH_b = dl/dG_b / sqrt(s) - (sum_a dl/dG_a H_a) / (2 s^1.5) ds/dH_b,  dH_N/do1 = fN (1 - tanh^2 o1).
__device__ __forceinline__ void fsai_chain(const float* st, const float* o, int64_t s, int64_t n, int64_t m, int64_t p,
                                           float dC, float dN, float dW, float* dout) {
  const float o1 = o ? o[s * 3 * n + n + p] : 0.f, o2 = o ? o[s * 3 * n + 2 * n + p] : 0.f;
  const FsaiRow fr = fsai_row(st + s * 5 * n, n, m, p, o1, o2);
  float hN_g = dN, hW_g = dW;
  if (o) {
    const float is = rsqrtf(fr.s);
    const float k = 0.5f * (dC * fr.hC + dN * fr.hN + dW * fr.hW) * is * is * is;
    hN_g = dN * is - k * 2.f * (fr.hN * fr.dN + fr.hC * fr.aN);
    hW_g = dW * is - k * 2.f * (fr.hW * fr.dW + fr.hC * fr.aW);
  }
  const float t1 = tanhf(o1), t2 = tanhf(o2);
  dout[s * 3 * n + p] = 0.f;
  dout[s * 3 * n + n + p] = hN_g * fr.fN * (1.f - t1 * t1);
  dout[s * 3 * n + 2 * n + p] = hW_g * fr.fW * (1.f - t2 * t2);
}

// ---- spectral (Rayleigh-quotient) loss -------------------------------------------------------
// For a pair (r = A e, e): R = (A e)^T P (A e) / e^T A e = |G r|^2 / e^T r, the Rayleigh quotient of
// P A in the A inner product.  loss = sum_s w_s log R_s with w_s = +1/#high for white-noise errors
// (the top of the spectrum) and -1/#low for the smooth errors PCG leaves behind (the bottom): a
// scale-free proxy of log cond(P A).  d log R / dG_pq = 2 t_p r_q / |t|^2 with t = G r.
// sc[s] = e^T r, sc[S + s] = |t|^2.
__global__ void __launch_bounds__(256) k_fsai_rq_t(const float* __restrict__ gs, const float* __restrict__ r,
                                                   const float* __restrict__ e, int64_t m, int64_t S,
                                                   float* __restrict__ t, double* sc) {
  __shared__ float red[32];
  const int64_t n = m * m;
  const int64_t s = blockIdx.y;
  const float* gss = gs + s * 3 * n;
  float er = 0.f, tt = 0.f;
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
    const float tv = g_row(gss, n, m, p, r + s * n);
    t[s * n + p] = tv;
    er += e[s * n + p] * r[s * n + p];
    tt += tv * tv;
  }
  er = block_sum(er, red);
  tt = block_sum(tt, red);
  if (threadIdx.x == 0) {
    atomicAdd(sc + s, (double)er);
    atomicAdd(sc + S + s, (double)tt);
  }
}

__global__ void k_fsai_rq_grad(const float* __restrict__ st, const float* __restrict__ o, const float* __restrict__ r,
                               const float* __restrict__ t, const double* __restrict__ sc,
                               const float* __restrict__ w, int64_t m, int64_t S, float* __restrict__ dout) {
  const int64_t n = m * m;
  const int64_t s = blockIdx.y;
  const float coef = (float)(2.0 * (double)w[s] / sc[S + s]);
  const float* rs = r + s * n;
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = p / m, j = p % m;
    const float ct = coef * t[s * n + p];
    const float dC = ct * rs[p];
    const float dN = i > 0 ? ct * rs[p - m] : 0.f;
    const float dW = j > 0 ? ct * rs[p - 1] : 0.f;
    fsai_chain(st, o, s, n, m, p, dC, dN, dW, dout);
  }
}

// t = G r ; sc[0] += e^T r
__global__ void __launch_bounds__(256) k_fsai_loss_t(const float* __restrict__ gs, const float* __restrict__ r,
                                                     const float* __restrict__ e, int64_t m, int64_t S,
                                                     float* __restrict__ t, double* sc) {
  __shared__ float red[32];
  const int64_t n = m * m;
  const int64_t s = blockIdx.y;
  const float* gss = gs + s * 3 * n;
  float acc = 0.f;
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
    t[s * n + p] = g_row(gss, n, m, p, r + s * n);
    acc += e[s * n + p] * r[s * n + p];
  }
  acc = block_sum(acc, red);
  if (threadIdx.x == 0) atomicAdd(sc + s, (double)acc);
}

// v = G^T t
__global__ void k_fsai_loss_v(const float* __restrict__ gs, const float* __restrict__ t, int64_t m, int64_t S,
                              float* __restrict__ v) {
  const int64_t n = m * m;
  const int64_t s = blockIdx.y;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x)
    v[s * n + q] = gt_row(gs + s * 3 * n, n, m, q, t + s * n);
}

// w = A v ; sc[1] += v^T w ; sc[2] += v^T r
__global__ void __launch_bounds__(256) k_fsai_loss_w(const float* __restrict__ st, const float* __restrict__ v,
                                                     const float* __restrict__ r, int64_t m, int64_t S,
                                                     float* __restrict__ w, double* sc) {
  __shared__ float red[32];
  const int64_t n = m * m;
  const int64_t s = blockIdx.y;
  float a1 = 0.f, a2 = 0.f;
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
    const float wv = a_row(st + s * 5 * n, n, m, p, v + s * n);
    w[s * n + p] = wv;
    a1 += v[s * n + p] * wv;
    a2 += v[s * n + p] * r[s * n + p];
  }
  a1 = block_sum(a1, red);
  a2 = block_sum(a2, red);
  if (threadIdx.x == 0) {
    atomicAdd(sc + S + s, (double)a1);
    atomicAdd(sc + 2 * S + s, (double)a2);
  }
}

// gradient w.r.t. the network output o (S, 3, m, m), averaged over systems
__global__ void k_fsai_loss_grad(const float* __restrict__ st, const float* __restrict__ o,
                                 const float* __restrict__ gs, const float* __restrict__ r, const float* __restrict__ t,
                                 const float* __restrict__ w, const double* __restrict__ sc, int64_t m, int64_t S,
                                 float* __restrict__ dout) {
  const int64_t n = m * m;
  const int64_t s = blockIdx.y;
  const float inv = (float)(2.0 / (sc[s] * (double)S));
  const float* rs = r + s * n;
  const float* ws = w + s * n;
  const float* gss = gs + s * 3 * n;
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = p / m, j = p % m;
    const float gp = inv * (ws[p] - rs[p]);
    const float gN = i > 0 ? inv * (ws[p - m] - rs[p - m]) : 0.f;
    const float gW = j > 0 ? inv * (ws[p - 1] - rs[p - 1]) : 0.f;
    const float GN = gss[p], GW = gss[n + p], GC = gss[2 * n + p];
    const float u = GC * gp + GN * gN + GW * gW;
    const float tp = t[s * n + p];
    const float dC = tp * gp + u * rs[p];
    const float dN = i > 0 ? tp * gN + u * rs[p - m] : 0.f;
    const float dW = j > 0 ? tp * gW + u * rs[p - 1] : 0.f;
    fsai_chain(st, o, s, n, m, p, dC, dN, dW, dout);
  }
}

// Adam (decoupled, no weight decay)
__global__ void k_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m1,
                       float* __restrict__ m2, int64_t count, float lr, float b1, float b2, float eps, float c1, float c2) {
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < count; q += (int64_t)gridDim.x * blockDim.x) {
    const float gv = g[q];
    const float a = b1 * m1[q] + (1.f - b1) * gv;
    const float b = b2 * m2[q] + (1.f - b2) * gv * gv;
    m1[q] = a;
    m2[q] = b;
    p[q] -= lr * (a / c1) / (sqrtf(b / c2) + eps);
  }
}

static int grid_for(int64_t total) {
  const int64_t want = ceil_div(total, 256);
  const int64_t cap = (int64_t)num_sms() * 16;
  return (int)(want < 1 ? 1 : (want > cap ? cap : want));
}

}  // namespace colagb

using namespace colagb;

extern "C" int colagb_grid5_stencil(const int32_t* indptr, const int32_t* indices, const float* values, int64_t nnz,
                                    int64_t m, int64_t S, float* stencil, int32_t* err_flag, void* stream) {
  if (!indptr || !indices || !values || !stencil || !err_flag || m < 1 || S < 0)
    return fail(COLAGB_ERR_INVALID, "colagb_grid5_stencil: bad arguments");
  if (S == 0) return COLAGB_OK;
  k_grid5_stencil<<<grid_for(S * m * m), 256, 0, as_stream(stream)>>>(indptr, indices, values, nnz, m, S, stencil,
                                                                      err_flag);
  COLAGB_CUDA(cudaGetLastError());
  return COLAGB_OK;
}

extern "C" int colagb_fsai_features(const float* stencil, int64_t m, int64_t S, float* feats, void* stream) {
  if (!stencil || !feats || m < 1 || S < 0) return fail(COLAGB_ERR_INVALID, "colagb_fsai_features: bad arguments");
  if (S == 0) return COLAGB_OK;
  k_fsai_features<<<grid_for(S * m * m), 256, 0, as_stream(stream)>>>(stencil, m, S, feats);
  COLAGB_CUDA(cudaGetLastError());
  return COLAGB_OK;
}

extern "C" int colagb_fsai_assemble(const float* stencil, const float* net_out, int64_t m, int64_t S, float* g_stencil,
                                    void* stream) {
  if (!stencil || !g_stencil || m < 1 || S < 0) return fail(COLAGB_ERR_INVALID, "colagb_fsai_assemble: bad arguments");
  if (S == 0) return COLAGB_OK;
  k_fsai_assemble<<<grid_for(S * m * m), 256, 0, as_stream(stream)>>>(stencil, net_out, m, S, g_stencil);
  COLAGB_CUDA(cudaGetLastError());
  return COLAGB_OK;
}

extern "C" int colagb_fsai_compact(const float* g_stencil, const int32_t* g_indptr, int64_t m, int64_t S, int64_t g_nnz,
                                   float* g_values, void* stream) {
  if (!g_stencil || !g_indptr || !g_values || m < 1 || S < 0)
    return fail(COLAGB_ERR_INVALID, "colagb_fsai_compact: bad arguments");
  if (S == 0) return COLAGB_OK;
  k_fsai_compact<<<grid_for(S * m * m), 256, 0, as_stream(stream)>>>(g_stencil, g_indptr, m, S, g_nnz, g_values);
  COLAGB_CUDA(cudaGetLastError());
  return COLAGB_OK;
}

extern "C" int colagb_fsai_net_build(const float* stencil, const float* params, int64_t n_params, int64_t m, int64_t S,
                                     const int32_t* g_indptr, int64_t g_nnz, float* g_values, uint32_t* tile_counter,
                                     void* stream) {
  if (!stencil || !params || !g_indptr || !g_values || m < 1 || S < 0)
    return fail(COLAGB_ERR_INVALID, "colagb_fsai_net_build: bad arguments");
  if (n_params != kNetParams)
    return fail(COLAGB_ERR_INVALID, "colagb_fsai_net_build: the network has " + std::to_string(kNetParams) +
                                        " parameters (6->16->16->3 3x3 convolutions), got " + std::to_string(n_params));
  if (S == 0) return COLAGB_OK;
  COLAGB_CUDA(cudaFuncSetAttribute(k_fsai_net_build, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kNetSmemBytes));
  const int64_t side = (m + kNetTile - 1) / kNetTile;
  const int64_t tiles = side * side * S;
  const int grid = (int)std::min<int64_t>(tiles, num_sms());
  if (tile_counter) COLAGB_CUDA(cudaMemsetAsync(tile_counter, 0, sizeof(uint32_t), as_stream(stream)));
  k_fsai_net_build<<<grid, kNetThreads, kNetSmemBytes, as_stream(stream)>>>(stencil, params, m, S, g_indptr, g_nnz,
                                                                            g_values, tile_counter);
  COLAGB_CUDA(cudaGetLastError());
  return COLAGB_OK;
}

extern "C" int colagb_fsai_closed_build(const float* stencil, int64_t m, int64_t S, const int32_t* g_indptr,
                                        int64_t g_nnz, float* g_values, void* stream) {
  if (!stencil || !g_indptr || !g_values || m < 1 || S < 0)
    return fail(COLAGB_ERR_INVALID, "colagb_fsai_closed_build: bad arguments");
  if (S == 0) return COLAGB_OK;
  k_fsai_closed_build<<<grid_for(S * m * m), 256, 0, as_stream(stream)>>>(stencil, m, S, g_indptr, g_nnz, g_values);
  COLAGB_CUDA(cudaGetLastError());
  return COLAGB_OK;
}

extern "C" int colagb_conv3x3_forward(const float* in, int64_t B, int32_t cin, int32_t cout, int64_t H, int64_t W,
                                      const float* weight, const float* bias, int32_t relu, float* out, void* stream) {
  if (!in || !weight || !out || B < 0 || cin < 1 || H < 1 || W < 1 || (cout != 16 && cout != 3))
    return fail(COLAGB_ERR_INVALID, "colagb_conv3x3_forward: bad arguments (cout must be 16 or 3)");
  if (B == 0) return COLAGB_OK;
  const size_t smem = (size_t)cout * cin * 9 * sizeof(float);
  if (smem > 40 * 1024) return fail(COLAGB_ERR_INVALID, "colagb_conv3x3_forward: too many weights");
  dim3 grid((unsigned)ceil_div(W, 16), (unsigned)ceil_div(H, 16), (unsigned)B);
  if (cout == 16)
    k_conv3_fwd<16><<<grid, 256, smem, as_stream(stream)>>>(in, cin, (int)H, (int)W, weight, bias, relu, out);
  else
    k_conv3_fwd<3><<<grid, 256, smem, as_stream(stream)>>>(in, cin, (int)H, (int)W, weight, bias, relu, out);
  COLAGB_CUDA(cudaGetLastError());
  return COLAGB_OK;
}

extern "C" int colagb_conv3x3_backward(const float* grad_out, const float* act, const float* in, int64_t B, int32_t cin,
                                       int32_t cout, int64_t H, int64_t W, const float* weight, float* grad_in,
                                       float* grad_wb, float* scratch, size_t scratch_bytes, void* stream) {
  if (!grad_out || !in || !weight || !grad_wb || B < 0 || cin < 1 || cout < 1 || H < 1 || W < 1)
    return fail(COLAGB_ERR_INVALID, "colagb_conv3x3_backward: bad arguments");
  if (grad_in && cin != 16 && cin != 6) return fail(COLAGB_ERR_INVALID, "colagb_conv3x3_backward: cin must be 16 or 6");
  const int nw = cout * cin * 9;
  if (nw > 12 * 256) return fail(COLAGB_ERR_INVALID, "colagb_conv3x3_backward: too many weights");
  cudaStream_t st = as_stream(stream);
  const int nblk = num_sms() * 2;
  const size_t need = (size_t)nblk * (nw + cout) * sizeof(float);
  if (!scratch || scratch_bytes < need)
    return fail(COLAGB_ERR_WORKSPACE, "colagb_conv3x3_backward: scratch too small (need " + std::to_string(need) + ")");
  if (B == 0) return COLAGB_OK;
  const size_t smw = (size_t)(cout * 256 + cin * 324) * sizeof(float);
  if (smw > 48 * 1024)
    COLAGB_CUDA(cudaFuncSetAttribute(k_conv3_bwd_weight, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smw));
  k_conv3_bwd_weight<<<nblk, 256, smw, st>>>(grad_out, act, in, (int)B, cin, cout, (int)H, (int)W, scratch);
  k_sum_partials<<<(unsigned)ceil_div(nw + cout, 256), 256, 0, st>>>(scratch, nblk, nw + cout, grad_wb, 0);
  if (grad_in) {
    const size_t sm = (size_t)nw * sizeof(float);
    dim3 grid((unsigned)ceil_div(W, 16), (unsigned)ceil_div(H, 16), (unsigned)B);
    if (cin == 16) k_conv3_bwd_data<16><<<grid, 256, sm, st>>>(grad_out, act, cout, (int)H, (int)W, weight, grad_in);
    else k_conv3_bwd_data<6><<<grid, 256, sm, st>>>(grad_out, act, cout, (int)H, (int)W, weight, grad_in);
  }
  COLAGB_CUDA(cudaGetLastError());
  return COLAGB_OK;
}

extern "C" int colagb_conv3x3_backward_scratch_bytes(int32_t cin, int32_t cout, size_t* bytes) {
  if (!bytes) return fail(COLAGB_ERR_INVALID, "null");
  *bytes = (size_t)num_sms() * 2 * (cout * cin * 9 + cout) * sizeof(float);
  return COLAGB_OK;
}

extern "C" int colagb_fsai_loss_grad(const float* stencil, const float* net_out, const float* g_stencil, const float* r,
                                     const float* e, int64_t m, int64_t S, float* grad_out, double* loss_terms,
                                     float* scratch, size_t scratch_bytes, void* stream) {
  if (!stencil || !g_stencil || !r || !e || !loss_terms || !scratch || m < 1 || S < 0)
    return fail(COLAGB_ERR_INVALID, "colagb_fsai_loss_grad: bad arguments");
  const int64_t n = m * m;
  const size_t need = (size_t)3 * S * n * sizeof(float);
  if (scratch_bytes < need) return fail(COLAGB_ERR_WORKSPACE, "colagb_fsai_loss_grad: scratch too small");
  if (S == 0) return COLAGB_OK;
  cudaStream_t st = as_stream(stream);
  float* t = scratch;
  float* v = t + S * n;
  float* w = v + S * n;
  COLAGB_CUDA(cudaMemsetAsync(loss_terms, 0, 3 * S * sizeof(double), st));
  dim3 grid((unsigned)std::min<int64_t>(ceil_div(n, 256), 1024), (unsigned)S);
  k_fsai_loss_t<<<grid, 256, 0, st>>>(g_stencil, r, e, m, S, t, loss_terms);
  k_fsai_loss_v<<<grid, 256, 0, st>>>(g_stencil, t, m, S, v);
  k_fsai_loss_w<<<grid, 256, 0, st>>>(stencil, v, r, m, S, w, loss_terms);
  if (grad_out) k_fsai_loss_grad<<<grid, 256, 0, st>>>(stencil, net_out, g_stencil, r, t, w, loss_terms, m, S, grad_out);
  COLAGB_CUDA(cudaGetLastError());
  return COLAGB_OK;
}

extern "C" int colagb_fsai_rq_loss_grad(const float* stencil, const float* net_out, const float* g_stencil,
                                        const float* r, const float* e, const float* weights, int64_t m, int64_t S,
                                        float* grad_out, double* loss_terms, float* scratch, size_t scratch_bytes,
                                        void* stream) {
  if (!stencil || !g_stencil || !r || !e || !weights || !loss_terms || !scratch || m < 1 || S < 0)
    return fail(COLAGB_ERR_INVALID, "colagb_fsai_rq_loss_grad: bad arguments");
  const int64_t n = m * m;
  if (scratch_bytes < (size_t)S * n * sizeof(float))
    return fail(COLAGB_ERR_WORKSPACE, "colagb_fsai_rq_loss_grad: scratch too small");
  if (S == 0) return COLAGB_OK;
  cudaStream_t st = as_stream(stream);
  COLAGB_CUDA(cudaMemsetAsync(loss_terms, 0, 2 * S * sizeof(double), st));
  dim3 grid((unsigned)std::min<int64_t>(ceil_div(n, 256), 1024), (unsigned)S);
  k_fsai_rq_t<<<grid, 256, 0, st>>>(g_stencil, r, e, m, S, scratch, loss_terms);
  if (grad_out) k_fsai_rq_grad<<<grid, 256, 0, st>>>(stencil, net_out, r, scratch, loss_terms, weights, m, S, grad_out);
  COLAGB_CUDA(cudaGetLastError());
  return COLAGB_OK;
}

extern "C" int colagb_adam_step(float* param, const float* grad, float* m1, float* m2, int64_t count, float lr, float beta1,
                                float beta2, float eps, int32_t step, void* stream) {
  if (!param || !grad || !m1 || !m2 || count < 0 || step < 1) return fail(COLAGB_ERR_INVALID, "colagb_adam_step: bad arguments");
  if (count == 0) return COLAGB_OK;
  const float c1 = 1.f - powf(beta1, (float)step), c2 = 1.f - powf(beta2, (float)step);
  k_adam<<<grid_for(count), 256, 0, as_stream(stream)>>>(param, grad, m1, m2, count, lr, beta1, beta2, eps, c1, c2);
  COLAGB_CUDA(cudaGetLastError());
  return COLAGB_OK;
}
