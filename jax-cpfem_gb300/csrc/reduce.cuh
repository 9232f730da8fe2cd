// Deterministic grid reductions: every block writes its partial sums to a fixed slot,
// the last block to finish (ticket from an atomic counter) adds the slots in index
// order.  With a fixed grid the result is bitwise reproducible from run to run.
#pragma once

#include "cpfem_common.cuh"

namespace cpfem {

template <int NV>
__device__ __forceinline__ void warp_sum(double (&v)[NV]) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1)
#pragma unroll
    for (int k = 0; k < NV; ++k) v[k] += __shfl_down_sync(0xffffffffu, v[k], off);
}

// Sum v over the block; the result is valid in thread 0.  smem: NV*32 doubles.
template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV], double* smem) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  warp_sum<NV>(v);
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < NV; ++k) smem[k * 32 + wid] = v[k];
  __syncthreads();
  if (wid == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) v[k] = (lane < nw) ? smem[k * 32 + lane] : 0.0;
    warp_sum<NV>(v);
  }
  __syncthreads();
}

// Publish this block's partials; returns true in every thread of the last block, whose
// thread 0 then holds the grid totals in v.  partials: NV*gridDim.x doubles.
template <int NV>
__device__ __forceinline__ bool grid_sum(double (&v)[NV], double* partials, unsigned int* counter,
                                         double* smem) {
  __shared__ bool is_last;
  block_sum<NV>(v, smem);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) partials[k * gridDim.x + blockIdx.x] = v[k];
    __threadfence();
    const unsigned int ticket = atomicAdd(counter, 1u);
    is_last = (ticket == gridDim.x - 1);
  }
  __syncthreads();
  if (!is_last) return false;
  __threadfence();
  double acc[NV];
#pragma unroll
  for (int k = 0; k < NV; ++k) acc[k] = 0.0;
  for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x)
#pragma unroll
    for (int k = 0; k < NV; ++k) acc[k] += __ldcg(&partials[k * gridDim.x + b]);
  block_sum<NV>(acc, smem);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) v[k] = acc[k];
    *counter = 0u;
  }
  return true;
}

}  // namespace cpfem
