// Operator programs: the LinearOperator tree of cola/ops/operators.py lowered to nodes that the
// host-side executor walks, launching one leaf kernel per Dense / Sparse / Diagonal / scalar node.
#pragma once

#include <vector>
#include "common.cuh"

struct colagb_op {
  std::vector<colagb_op_node> nodes;           // copy of the caller's nodes
  std::vector<std::vector<int32_t>> children;  // copied child index lists
  std::vector<std::vector<int64_t>> mult;      // copied multiplicities (BLOCKDIAG)
  int32_t root = 0;
  int32_t compute_dtype = COLAGB_F32;
};

namespace colagb {

// Y[b] = alpha * op(X[b]) + beta * Y[b] for b < batch; X[b] = X + b * bsx, Y[b] = Y + b * bsy.
// T is the compute type (float or double).  `skip` (device, may be null): when *skip != 0
// every leaf kernel returns at once (used to make over-scheduled CG iterations free).
template <class T>
int op_apply(const colagb_op* op, int node, const T* X, int64_t ldx, int64_t bsx, T* Y, int64_t ldy,
             int64_t bsy, int64_t k, int64_t batch, T alpha, T beta, Bump& ws, const int* skip,
             cudaStream_t st);

// Leaf kernels exposed to the solvers.
template <class T>
int launch_axpby(const T* X, int64_t ldx, T* Y, int64_t ldy, int64_t rows, int64_t k, T alpha, T beta,
                 const int* skip, cudaStream_t st);

// Whether the operator is a single CSR or Dense leaf, optionally plus a scalar shift
// (Sum(leaf, ScalarMul) or Sum(leaf, Identity)), i.e. what the fused persistent CG handles.
struct FusedForm {
  bool ok = false;
  const colagb_op_node* leaf = nullptr;
  double shift = 0.0;
};
FusedForm fused_form(const colagb_op* op);

// Tensor-core factor contraction of the Kronecker matvec (tc_gemm.cu):
// out[b * s_b + m * s_m + n * s_n] = alpha * sum_k A_b[m, k] B[n, k] + beta * out[...], with
// A_b[m, k] = a_src[b * K * M + k * M + m] (transposed_a) or A[m, k] = a_src[m * K + k] (batch 1),
// B[n, k] = b_src[n * ldb + k].  BF16 products with FP32 accumulation; `split` adds the lo terms of
// the three-product BF16 split.  Scratch is taken from ws (sizes only when ws.measure).
bool tc_contract_supported(int64_t batch, int64_t M, int64_t N, int64_t K);
int tc_contract(const float* a_src, bool transposed_a, int64_t batch, int64_t M, int64_t K, const void* b_src,
                int32_t b_dtype, int64_t ldb, int64_t N, float* out, int64_t s_b, int64_t s_m, int64_t s_n,
                float alpha, float beta, bool split, Bump& ws, const int* skip, cudaStream_t st);

}  // namespace colagb
