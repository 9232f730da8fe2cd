// FP64 throughput probe: the denominator of the FP64 rooflines.
// Every thread runs 16 independent FMA chains, unrolled 4 deep inside a 32-bit loop (64
// FMAs per loop trip: the loop's integer and branch instructions are a few percent of the
// issue slots); the grid fills every SM at full occupancy, several times over.
#include "cpfem_common.cuh"

namespace cpfem {

constexpr int kProbeChains = 16;

__global__ void __launch_bounds__(256) k_dfma_probe(int32_t iters, double seed, double* out) {
  double a[kProbeChains];
#pragma unroll
  for (int k = 0; k < kProbeChains; ++k) a[k] = seed + 1e-3 * (threadIdx.x + k);
  const double m = 0.999999, c = 1e-7;
  for (int32_t i = 0; i < iters; ++i) {
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int k = 0; k < kProbeChains; ++k) a[k] = fma(a[k], m, c);
  }
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < kProbeChains; ++k) s += a[k];
  if (s == 12345.678) out[0] = s;  // keeps the chains live
}

}  // namespace cpfem

extern "C" int cpfem_probe_dfma(int64_t iters, int32_t blocks, double* out, double* flops, void* stream) {
  CPFEM_REQUIRE(iters > 0 && iters <= (1 << 30) && blocks > 0 && out != nullptr && flops != nullptr,
                "bad probe arguments");
  cpfem::k_dfma_probe<<<blocks, 256, 0, (cudaStream_t)stream>>>((int32_t)iters, 1.0, out);
  CPFEM_CUDA_TRY(cudaGetLastError());
  *flops = 2.0 * 4.0 * cpfem::kProbeChains * (double)iters * 256.0 * (double)blocks;
  return CPFEM_OK;
}
