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

}  // namespace colagb
