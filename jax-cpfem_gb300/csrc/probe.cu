// FP64 throughput probe: the denominator of the constitutive kernel's roofline.
// Each thread runs 8 independent FMA chains, enough to cover the FP64 pipe latency;
// the grid covers every SM several times.
#include "cpfem_common.cuh"

namespace cpfem {

__global__ void __launch_bounds__(256) k_dfma_probe(int64_t iters, double seed, double* out) {
  double a[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) a[k] = seed + 1e-3 * (threadIdx.x + k);
  const double m = 0.999999, c = 1e-7;
  for (int64_t i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = fma(a[k], m, c);
  }
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += a[k];
  if (s == 12345.678) out[0] = s;  // keeps the chains live
}

}  // namespace cpfem

extern "C" int cpfem_probe_dfma(int64_t iters, int32_t blocks, double* out, double* flops, void* stream) {
  CPFEM_REQUIRE(iters > 0 && blocks > 0 && out != nullptr && flops != nullptr, "bad probe arguments");
  cpfem::k_dfma_probe<<<blocks, 256, 0, (cudaStream_t)stream>>>(iters, 1.0, out);
  CPFEM_CUDA_TRY(cudaGetLastError());
  *flops = 2.0 * 8.0 * (double)iters * 256.0 * (double)blocks;
  return CPFEM_OK;
}
