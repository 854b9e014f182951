// Thread-block-cluster helpers shared by the cluster schedules of the batched PCG.
#pragma once

#include <cooperative_groups.h>

#include "common.cuh"

namespace colagb {

// Cluster-wide sums of NQ values: CTA partials go to this CTA's `slot`, a cluster barrier publishes
// them, and every CTA adds all ranks' slots in rank order, so every CTA of the cluster derives
// bit-identical sums.  Callers alternate `slot` between two buffers: a CTA only overwrites a buffer
// after the next cluster barrier, by which time every reader of the previous round has finished.
template <int NQ, int CL>
__device__ __forceinline__ void cluster_sum(cooperative_groups::cluster_group& cl, double (&v)[NQ], double* slot,
                                            double* red, double* bcast) {
#pragma unroll
  for (int k = 0; k < NQ; ++k) {
    const double x = block_sum(v[k], red);
    if (threadIdx.x == 0) slot[k] = x;
  }
  cl.sync();
  if (threadIdx.x < NQ) {
    double s = 0.0;
#pragma unroll
    for (int r = 0; r < CL; ++r) s += *cl.map_shared_rank(slot + threadIdx.x, r);
    bcast[threadIdx.x] = s;
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < NQ; ++k) v[k] = bcast[k];
  __syncthreads();
}

// Split cluster barrier: arrive (release) publishes this thread's prior writes, wait (acquire)
// returns once every thread of the cluster has arrived.  Work placed between the two overlaps the
// barrier's latency.  Every thread must call them in strict arrive / wait alternation.
__device__ __forceinline__ void cluster_arrive() { asm volatile("barrier.cluster.arrive.release.aligned;\n" ::: "memory"); }
__device__ __forceinline__ void cluster_wait() { asm volatile("barrier.cluster.wait.acquire.aligned;\n" ::: "memory"); }

// FP32 cluster-wide sums for the per-iteration inner products, built for latency: a butterfly in
// each warp, one block barrier, then warp 0 of every CTA stores the CTA's totals straight into every
// peer's `slot` (distributed shared memory, entry [q][rank]), one cluster barrier publishes them,
// and every warp reads the CL partials from its own shared memory and combines them with the same
// butterfly.  Every thread of every CTA ends with bit-identical sums (the same values in the same
// lanes, fixed combination order; a + b == b + a in IEEE arithmetic).  `wpart` holds NQ x 32
// floats; `slot` NQ x CL floats and must alternate between two buffers across consecutive calls: a
// CTA writes a peer's buffer again only two calls later, after the intervening cluster barrier that
// the peer reaches once it has read that buffer.
template <int NQ, int CL>
__device__ __forceinline__ void cluster_sum_f(cooperative_groups::cluster_group& cl, float (&v)[NQ], float* wpart,
                                              float* slot) {
  static_assert(CL <= 32, "one warp combines the CTA partials");
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nw = blockDim.x >> 5;
#pragma unroll
  for (int q = 0; q < NQ; ++q) {
    const float x = warp_sum(v[q]);
    if (lane == 0) wpart[q * 32 + warp] = x;
  }
  __syncthreads();
  if (warp == 0) {
    const int rank = (int)cl.block_rank();
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
      const float x = warp_sum(lane < nw ? wpart[q * 32 + lane] : 0.f);  // every lane holds the total
      if (lane < CL) *cl.map_shared_rank(slot + q * CL + rank, lane) = x;
    }
  }
  cl.sync();
#pragma unroll
  for (int q = 0; q < NQ; ++q) v[q] = warp_sum(lane < CL ? slot[q * CL + lane] : 0.f);
}

// cluster_sum_f in two halves, so that work which does not need the sums runs while the cluster
// barrier completes: _begin publishes this CTA's partials into every peer and arrives on the
// barrier (release), _end waits on it (acquire) and combines.  Same results as cluster_sum_f.
template <int NQ, int CL>
__device__ __forceinline__ void cluster_sum_f_begin(cooperative_groups::cluster_group& cl, float (&v)[NQ],
                                                    float* wpart, float* slot) {
  static_assert(CL <= 32, "one warp combines the CTA partials");
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nw = blockDim.x >> 5;
#pragma unroll
  for (int q = 0; q < NQ; ++q) {
    const float x = warp_sum(v[q]);
    if (lane == 0) wpart[q * 32 + warp] = x;
  }
  __syncthreads();
  if (warp == 0) {
    const int rank = (int)cl.block_rank();
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
      const float x = warp_sum(lane < nw ? wpart[q * 32 + lane] : 0.f);
      if (lane < CL) *cl.map_shared_rank(slot + q * CL + rank, lane) = x;
    }
  }
  cluster_arrive();
}

template <int NQ, int CL>
__device__ __forceinline__ void cluster_sum_f_end(float (&v)[NQ], const float* slot) {
  const int lane = threadIdx.x & 31;
  cluster_wait();
#pragma unroll
  for (int q = 0; q < NQ; ++q) v[q] = warp_sum(lane < CL ? slot[q * CL + lane] : 0.f);
}

}  // namespace colagb
