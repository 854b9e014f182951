// Vector-Jacobian products of the structured matvec with respect to the operator's own tensors:
// for Y = op(theta) X and a cotangent G, grad_theta += alpha * d<G, op(theta) X>/d theta.
//
// The reference takes these through autograd of the operator's _matmat (cg_bwd, cola/linalg/inverse/
// cg.py:72-86, and slq_bwd, cola/linalg/tbd/slq.py:10-31, differentiate A(theta) @ x in its backend).
// Here they are kernels on the device, for the leaves and the compositions whose VJP needs no
// intermediate products:
//   Dense     dA[i][j]   += alpha * sum_c G[i, c] X[j, c]       (a k-term outer product per entry)
//   Sparse    dvals[e]   += alpha * sum_c G[row(e), c] X[col(e), c]
//   Diagonal  dd[i]      += alpha * sum_c G[i, c] X[i, c]
//   Sum       each child with the same G and X; ScalarMul / Identity have no tensors.
// Product, Kronecker and BlockDiag trees return COLAGB_ERR_UNSUPPORTED (the caller differentiates
// those through a tensor-op restatement).
#include "common.cuh"
#include "ops.cuh"

namespace colagb {

template <class T>
__global__ void k_vjp_dense(T* __restrict__ dA, int64_t rows, int64_t cols, const T* __restrict__ X, int64_t ldx,
                            const T* __restrict__ G, int64_t ldg, int64_t k, T alpha) {
  const int64_t total = rows * cols;
  for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < total; u += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = u / cols, j = u - i * cols;
    T acc = T(0);
    for (int64_t c = 0; c < k; ++c) acc += G[i * ldg + c] * X[j * ldx + c];
    dA[u] += alpha * acc;
  }
}

template <class T>
__global__ void k_vjp_csr(T* __restrict__ dv, const int32_t* __restrict__ indptr, const int32_t* __restrict__ indices,
                          int64_t rows, const T* __restrict__ X, int64_t ldx, const T* __restrict__ G, int64_t ldg,
                          int64_t k, T alpha) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < rows; i += (int64_t)gridDim.x * blockDim.x) {
    for (int32_t e = indptr[i]; e < indptr[i + 1]; ++e) {
      const int64_t j = indices[e];
      T acc = T(0);
      for (int64_t c = 0; c < k; ++c) acc += G[i * ldg + c] * X[j * ldx + c];
      dv[e] += alpha * acc;
    }
  }
}

template <class T>
__global__ void k_vjp_diag(T* __restrict__ dd, int64_t rows, const T* __restrict__ X, int64_t ldx,
                           const T* __restrict__ G, int64_t ldg, int64_t k, T alpha) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < rows; i += (int64_t)gridDim.x * blockDim.x) {
    T acc = T(0);
    for (int64_t c = 0; c < k; ++c) acc += G[i * ldg + c] * X[i * ldx + c];
    dd[i] += alpha * acc;
  }
}

static int vjp_supported(const colagb_op* op, int node) {
  const colagb_op_node& nd = op->nodes[node];
  switch (nd.kind) {
    case COLAGB_OP_DENSE:
    case COLAGB_OP_CSR:
    case COLAGB_OP_DIAG:
      if (nd.dtype == COLAGB_BF16) return fail(COLAGB_ERR_UNSUPPORTED, "matmat VJP: BF16 leaves have no gradient here");
      if (nd.perm) return fail(COLAGB_ERR_UNSUPPORTED, "matmat VJP: permuted Sparse leaves are not handled");
      return COLAGB_OK;
    case COLAGB_OP_SCALAR:
    case COLAGB_OP_IDENTITY:
      return COLAGB_OK;
    case COLAGB_OP_SUM:
      for (int32_t c : op->children[node]) COLAGB_TRY(vjp_supported(op, c));
      return COLAGB_OK;
    default:
      return fail(COLAGB_ERR_UNSUPPORTED, "matmat VJP: Product / Kronecker / BlockDiag trees are not handled");
  }
}

template <class T>
static int vjp_apply(const colagb_op* op, int node, const T* X, int64_t ldx, const T* G, int64_t ldg, int64_t k,
                     T alpha, void* const* grads, cudaStream_t st) {
  const colagb_op_node& nd = op->nodes[node];
  const int blocks = num_sms() * 8;
  if (nd.kind == COLAGB_OP_SUM) {
    for (int32_t c : op->children[node]) COLAGB_TRY(vjp_apply<T>(op, c, X, ldx, G, ldg, k, alpha, grads, st));
    return COLAGB_OK;
  }
  T* g = grads ? static_cast<T*>(grads[node]) : nullptr;
  if (!g || nd.rows == 0) return COLAGB_OK;
  if ((nd.dtype == COLAGB_F64) != std::is_same<T, double>::value)
    return fail(COLAGB_ERR_UNSUPPORTED, "matmat VJP: leaf storage type differs from the compute type");
  switch (nd.kind) {
    case COLAGB_OP_DENSE:
      if (nd.ld != nd.cols) return fail(COLAGB_ERR_UNSUPPORTED, "matmat VJP: Dense leaf with a row stride");
      k_vjp_dense<T><<<blocks, 256, 0, st>>>(g, nd.rows, nd.cols, X, ldx, G, ldg, k, alpha);
      break;
    case COLAGB_OP_CSR:
      k_vjp_csr<T><<<blocks, 256, 0, st>>>(g, nd.indptr, nd.indices, nd.rows, X, ldx, G, ldg, k, alpha);
      break;
    case COLAGB_OP_DIAG:
      k_vjp_diag<T><<<blocks, 256, 0, st>>>(g, nd.rows, X, ldx, G, ldg, k, alpha);
      break;
    default:
      return COLAGB_OK;
  }
  COLAGB_CUDA(cudaGetLastError());
  return COLAGB_OK;
}

}  // namespace colagb

using namespace colagb;

extern "C" int colagb_matmat_vjp(const colagb_op* op, const void* X, int64_t ldx, const void* G, int64_t ldg,
                                 int64_t k, double alpha, void* const* node_grads, void* stream) {
  if (!op || k < 0 || ldx < k || ldg < k) return fail(COLAGB_ERR_INVALID, "colagb_matmat_vjp: bad arguments");
  const colagb_op_node& r = op->nodes[op->root];
  if ((r.cols * k > 0 && !X) || (r.rows * k > 0 && !G)) return fail(COLAGB_ERR_INVALID, "colagb_matmat_vjp: null X/G");
  COLAGB_TRY(vjp_supported(op, op->root));
  cudaStream_t st = as_stream(stream);
  if (op->compute_dtype == COLAGB_F64)
    return vjp_apply<double>(op, op->root, static_cast<const double*>(X), ldx, static_cast<const double*>(G), ldg, k,
                             alpha, node_grads, st);
  return vjp_apply<float>(op, op->root, static_cast<const float*>(X), ldx, static_cast<const float*>(G), ldg, k,
                          (float)alpha, node_grads, st);
}
