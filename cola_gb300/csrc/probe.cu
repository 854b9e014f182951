// Read-bandwidth probe: the denominator of an honest roofline for kernels whose operands are served
// by L2 rather than HBM.
//
// The on-chip batched CG kernel re-reads each system's matrix diagonals from L2 at every step (the
// working set of the systems in flight, ~62 MB, stays in the 126 MB L2), so the HBM copy bandwidth
// is the wrong peak for it.  This kernel streams a caller buffer `reps` times with 128-bit loads
// that bypass L1 (ld.global.cg), every CTA reading a disjoint slice, and reduces the words so the
// loads cannot be dropped.  With a buffer that fits in L2 and reps >= 2, the time of the repeated
// passes is an L2 -> SM read bandwidth; with a buffer far larger than L2 it is an HBM read bandwidth.
#include "common.cuh"

namespace colagb {

__global__ void __launch_bounds__(512) k_read_stream(const float4* __restrict__ p, int64_t n4, int reps,
                                                     float* __restrict__ sink) {
  float acc = 0.f;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int r = 0; r < reps; ++r) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    // four independent loads in flight per thread per round
    for (; i + 3 * stride < n4; i += 4 * stride) {
      const float4 a = __ldcg(p + i), b = __ldcg(p + i + stride), c = __ldcg(p + i + 2 * stride),
                   d = __ldcg(p + i + 3 * stride);
      acc += (a.x + a.y + a.z + a.w) + (b.x + b.y + b.z + b.w) + (c.x + c.y + c.z + c.w) + (d.x + d.y + d.z + d.w);
    }
    for (; i < n4; i += stride) {
      const float4 a = __ldcg(p + i);
      acc += a.x + a.y + a.z + a.w;
    }
  }
  acc = warp_sum(acc);
  if ((threadIdx.x & 31) == 0 && acc == 1.2345678e30f) sink[0] = acc;  // never true for probe data
}

}  // namespace colagb

using namespace colagb;

extern "C" int colagb_read_bandwidth_probe(const void* buffer, size_t bytes, int32_t reps, void* sink, void* stream) {
  if (!buffer || !sink || reps < 1 || bytes < 16 || ((uintptr_t)buffer % 16) != 0)
    return fail(COLAGB_ERR_INVALID, "colagb_read_bandwidth_probe: bad arguments");
  const int64_t n4 = (int64_t)(bytes / 16);
  const int blocks = num_sms() * 4;
  k_read_stream<<<blocks, 512, 0, as_stream(stream)>>>(static_cast<const float4*>(buffer), n4, reps,
                                                       static_cast<float*>(sink));
  COLAGB_CUDA(cudaGetLastError());
  return COLAGB_OK;
}
