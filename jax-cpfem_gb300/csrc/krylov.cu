// Node-block SpMV and BiCGSTAB of the cpfem_gb300 C ABI.
//
// The matrix is the scalar CSR that scipy builds from the element COO triplets
// (crystal_plasticity_OR_design/solver.py:279-282), read through its node structure:
// rows 3a..3a+2 share node a's sorted neighbour list, so one warp reads the three rows
// with a single column list.  All BiCGSTAB scalars live on the device; every kernel
// of an iteration returns at once when the solve has finished, and the host only looks
// at the finished flag every check_every iterations.
#include <algorithm>

#include "cpfem_common.cuh"
#include "reduce.cuh"

namespace cpfem {

constexpr int kSpmvThreads = 256;
constexpr int kSpmvBlocks = 6 * 152;
constexpr int kMaxBlocks = 1024;   // partial-sum slots per reduced value

struct KState {
  double rho, rho_new, alpha, omega, atol2, rs;
  int k, done, exit_early, maxiter;
  unsigned int counter;
};

struct KWork {
  KState* st;
  double* partials;   // 8 * kMaxBlocks
  double *r, *rhat, *p, *q, *s, *t, *phat, *shat, *minv;
};

static size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

static size_t carve(void* base, int64_t n_nodes, KWork* w) {
  const int64_t n = 3 * n_nodes;
  char* p = (char*)base;
  size_t off = 0;
  auto take = [&](size_t bytes) {
    char* q = p ? p + off : nullptr;
    off += align256(bytes);
    return q;
  };
  KWork tmp;
  tmp.st = (KState*)take(sizeof(KState));
  tmp.partials = (double*)take(sizeof(double) * 8 * kMaxBlocks);
  double** vecs[] = {&tmp.r, &tmp.rhat, &tmp.p, &tmp.q, &tmp.s, &tmp.t, &tmp.phat, &tmp.shat};
  for (double** v : vecs) *v = (double*)take(sizeof(double) * n);
  tmp.minv = (double*)take(sizeof(double) * 9 * n_nodes);
  if (w) *w = tmp;
  return off;
}

// y(3 rows of node a) = A x or A^T x, summed over the warp (valid in every lane).
template <bool TRANS>
__device__ __forceinline__ void spmv_node(int64_t a, int lane, const int32_t* __restrict__ nrp,
                                          const int32_t* __restrict__ ncol, const int32_t* __restrict__ ntpos,
                                          const double* __restrict__ vals, const double* __restrict__ x,
                                          double* acc) {
  const int64_t r0 = nrp[a];
  const int64_t deg = nrp[a + 1] - r0;
  const int64_t rowlen = 3 * deg;
  acc[0] = acc[1] = acc[2] = 0.0;
  if (!TRANS) {
    const double* v0 = vals + 9 * r0;
    for (int64_t v = lane; v < rowlen; v += 32) {
      const int64_t j = v / 3;
      const int64_t k = v - 3 * j;
      const double xv = __ldg(&x[3 * (int64_t)__ldg(&ncol[r0 + j]) + k]);
      acc[0] = fma(__ldg(&v0[v]), xv, acc[0]);
      acc[1] = fma(__ldg(&v0[rowlen + v]), xv, acc[1]);
      acc[2] = fma(__ldg(&v0[2 * rowlen + v]), xv, acc[2]);
    }
  } else {
    for (int64_t v = lane; v < rowlen; v += 32) {
      const int64_t j = v / 3;
      const int64_t k = v - 3 * j;
      const int64_t b = __ldg(&ncol[r0 + j]);
      const int64_t rb = __ldg(&nrp[b]);
      const int64_t degb = __ldg(&nrp[b + 1]) - rb;
      const int64_t idx = 9 * rb + k * 3 * degb + 3 * (int64_t)__ldg(&ntpos[r0 + j]);
      const double xv = __ldg(&x[3 * b + k]);
      acc[0] = fma(__ldg(&vals[idx + 0]), xv, acc[0]);
      acc[1] = fma(__ldg(&vals[idx + 1]), xv, acc[1]);
      acc[2] = fma(__ldg(&vals[idx + 2]), xv, acc[2]);
    }
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1)
#pragma unroll
    for (int i = 0; i < 3; ++i) acc[i] += __shfl_xor_sync(0xffffffffu, acc[i], off);
}

template <bool TRANS>
__global__ void __launch_bounds__(kSpmvThreads) k_spmv(int32_t n_nodes, const int32_t* __restrict__ nrp,
                                                       const int32_t* __restrict__ ncol,
                                                       const int32_t* __restrict__ ntpos,
                                                       const double* __restrict__ vals,
                                                       const double* __restrict__ x, double* __restrict__ y) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t a = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); a < n_nodes; a += warps) {
    double acc[3];
    spmv_node<TRANS>(a, lane, nrp, ncol, ntpos, vals, x, acc);
    if (lane < 3) y[3 * a + lane] = acc[lane];
  }
}

// Diagonal (precond 1) or inverted 3x3 diagonal block (precond 2) per node.
template <bool TRANS>
__global__ void k_precond_setup(int32_t n_nodes, const int32_t* __restrict__ nrp, const int32_t* __restrict__ ncol,
                                const double* __restrict__ vals, int precond, double* __restrict__ minv) {
  const int64_t a = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= n_nodes) return;
  const int64_t r0 = nrp[a];
  const int64_t deg = nrp[a + 1] - r0;
  int64_t ja = -1;
  for (int64_t j = 0; j < deg; ++j)
    if (ncol[r0 + j] == a) ja = j;
  double blk[9];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const double v = (ja >= 0) ? vals[9 * r0 + i * 3 * deg + 3 * ja + k] : 0.0;
      if (TRANS) blk[3 * k + i] = v; else blk[3 * i + k] = v;
    }
  if (precond == 1) {
#pragma unroll
    for (int i = 0; i < 3; ++i) minv[3 * a + i] = 1.0 / blk[4 * i];
  } else {
    double bi[9];
    inv3(blk, bi);
#pragma unroll
    for (int c = 0; c < 9; ++c) minv[9 * a + c] = bi[c];
  }
}

__device__ __forceinline__ void apply_m(int precond, const double* __restrict__ minv, int64_t a,
                                        const double* v, double* out) {
  if (precond == 0) {
    out[0] = v[0]; out[1] = v[1]; out[2] = v[2];
  } else if (precond == 1) {
#pragma unroll
    for (int i = 0; i < 3; ++i) out[i] = v[i] * minv[3 * a + i];
  } else {
    const double* bi = minv + 9 * a;
#pragma unroll
    for (int i = 0; i < 3; ++i) out[i] = fma(bi[3 * i], v[0], fma(bi[3 * i + 1], v[1], bi[3 * i + 2] * v[2]));
  }
}

// r = b - A x0; rhat = p = q = r; scalars as jax's bicgstab initialises them.
template <bool TRANS>
__global__ void __launch_bounds__(kSpmvThreads) k_bicg_init(int32_t n_nodes, const int32_t* __restrict__ nrp,
                                                            const int32_t* __restrict__ ncol,
                                                            const int32_t* __restrict__ ntpos,
                                                            const double* __restrict__ vals,
                                                            const double* __restrict__ b,
                                                            const double* __restrict__ x, KWork w,
                                                            double tol, double atol) {
  __shared__ double smem[2 * 32];
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  double v[2] = {0.0, 0.0};
  for (int64_t a = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); a < n_nodes; a += warps) {
    double acc[3];
    spmv_node<TRANS>(a, lane, nrp, ncol, ntpos, vals, x, acc);
    if (lane < 3) {
      const int64_t d = 3 * a + lane;
      const double bv = b[d];
      const double rv = bv - acc[lane];
      w.r[d] = rv; w.rhat[d] = rv; w.p[d] = rv; w.q[d] = rv;
      v[0] = fma(bv, bv, v[0]);
      v[1] = fma(rv, rv, v[1]);
    }
  }
  if (grid_sum<2>(v, w.partials, &w.st->counter, smem) && threadIdx.x == 0) {
    KState* st = w.st;
    st->atol2 = fmax(tol * tol * v[0], atol * atol);
    st->rs = v[1];
    st->rho_new = v[1];
    st->rho = st->alpha = st->omega = 1.0;
    st->k = 0;
    st->exit_early = 0;
    st->done = !(st->rs > st->atol2 && 0 < st->maxiter);
  }
}

// p = r + beta (p - omega q); phat = M p
__global__ void __launch_bounds__(kVecThreads) k_bicg_p(int32_t n_nodes, KWork w, int precond) {
  const KState* st = w.st;
  if (__ldcg(&st->done)) return;
  const double beta = __ldcg(&st->rho_new) / __ldcg(&st->rho) * __ldcg(&st->alpha) / __ldcg(&st->omega);
  const double omega = __ldcg(&st->omega);
  for (int64_t a = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; a < n_nodes; a += (int64_t)gridDim.x * blockDim.x) {
    double pv[3], ph[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      const int64_t d = 3 * a + i;
      pv[i] = w.r[d] + beta * (w.p[d] - omega * w.q[d]);
      w.p[d] = pv[i];
    }
    apply_m(precond, w.minv, a, pv, ph);
#pragma unroll
    for (int i = 0; i < 3; ++i) w.phat[3 * a + i] = ph[i];
  }
}

// q = A phat ; alpha = rho_new / (rhat . q)
template <bool TRANS>
__global__ void __launch_bounds__(kSpmvThreads) k_bicg_q(int32_t n_nodes, const int32_t* __restrict__ nrp,
                                                         const int32_t* __restrict__ ncol,
                                                         const int32_t* __restrict__ ntpos,
                                                         const double* __restrict__ vals, KWork w) {
  __shared__ double smem[32];
  if (__ldcg(&w.st->done)) return;
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  double v[1] = {0.0};
  for (int64_t a = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); a < n_nodes; a += warps) {
    double acc[3];
    spmv_node<TRANS>(a, lane, nrp, ncol, ntpos, vals, w.phat, acc);
    if (lane < 3) {
      const int64_t d = 3 * a + lane;
      w.q[d] = acc[lane];
      v[0] = fma(w.rhat[d], acc[lane], v[0]);
    }
  }
  if (grid_sum<1>(v, w.partials, &w.st->counter, smem) && threadIdx.x == 0)
    w.st->alpha = w.st->rho_new / v[0];
}

// s = r - alpha q ; shat = M s ; exit_early = (s.s < atol2)
__global__ void __launch_bounds__(kVecThreads) k_bicg_s(int32_t n_nodes, KWork w, int precond) {
  __shared__ double smem[32];
  if (__ldcg(&w.st->done)) return;
  const double alpha = __ldcg(&w.st->alpha);
  double v[1] = {0.0};
  for (int64_t a = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; a < n_nodes; a += (int64_t)gridDim.x * blockDim.x) {
    double sv[3], sh[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      const int64_t d = 3 * a + i;
      sv[i] = w.r[d] - alpha * w.q[d];
      w.s[d] = sv[i];
      v[0] = fma(sv[i], sv[i], v[0]);
    }
    apply_m(precond, w.minv, a, sv, sh);
#pragma unroll
    for (int i = 0; i < 3; ++i) w.shat[3 * a + i] = sh[i];
  }
  if (grid_sum<1>(v, w.partials, &w.st->counter, smem) && threadIdx.x == 0)
    w.st->exit_early = (v[0] < w.st->atol2) ? 1 : 0;
}

// t = A shat ; omega = (t.s)/(t.t)
template <bool TRANS>
__global__ void __launch_bounds__(kSpmvThreads) k_bicg_t(int32_t n_nodes, const int32_t* __restrict__ nrp,
                                                         const int32_t* __restrict__ ncol,
                                                         const int32_t* __restrict__ ntpos,
                                                         const double* __restrict__ vals, KWork w) {
  __shared__ double smem[2 * 32];
  if (__ldcg(&w.st->done)) return;
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  double v[2] = {0.0, 0.0};
  for (int64_t a = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); a < n_nodes; a += warps) {
    double acc[3];
    spmv_node<TRANS>(a, lane, nrp, ncol, ntpos, vals, w.shat, acc);
    if (lane < 3) {
      const int64_t d = 3 * a + lane;
      w.t[d] = acc[lane];
      v[0] = fma(acc[lane], w.s[d], v[0]);
      v[1] = fma(acc[lane], acc[lane], v[1]);
    }
  }
  if (grid_sum<2>(v, w.partials, &w.st->counter, smem) && threadIdx.x == 0) w.st->omega = v[0] / v[1];
}

// x and r update, then the loop condition of jax's bicgstab for the next iteration.
__global__ void __launch_bounds__(kVecThreads) k_bicg_x(int32_t n_nodes, KWork w, double* __restrict__ x) {
  __shared__ double smem[2 * 32];
  if (__ldcg(&w.st->done)) return;
  const double alpha = __ldcg(&w.st->alpha);
  const double omega = __ldcg(&w.st->omega);
  const bool early = __ldcg(&w.st->exit_early) != 0;
  double v[2] = {0.0, 0.0};
  for (int64_t d = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; d < 3 * (int64_t)n_nodes;
       d += (int64_t)gridDim.x * blockDim.x) {
    double rv;
    if (early) {
      x[d] = x[d] + alpha * w.phat[d];
      rv = w.s[d];
    } else {
      x[d] = x[d] + (alpha * w.phat[d] + omega * w.shat[d]);
      rv = w.s[d] - omega * w.t[d];
    }
    w.r[d] = rv;
    v[0] = fma(rv, rv, v[0]);
    v[1] = fma(w.rhat[d], rv, v[1]);
  }
  if (grid_sum<2>(v, w.partials, &w.st->counter, smem) && threadIdx.x == 0) {
    KState* st = w.st;
    int k = (st->omega == 0.0 || st->alpha == 0.0) ? -11 : st->k + 1;
    if (st->rho_new == 0.0) k = -10;
    st->k = k;
    st->rho = st->rho_new;
    st->rho_new = v[1];
    st->rs = v[0];
    st->done = !(st->rs > st->atol2 && k < st->maxiter && k >= 0);
  }
}

template <bool TRANS>
static int run_bicgstab(int32_t n_nodes, const int32_t* nrp, const int32_t* ncol, const int32_t* ntpos,
                        const double* vals, const double* b, double* x, int precond, double tol, double atol,
                        int32_t maxiter, int32_t check_every, void* workspace, int32_t* info, cudaStream_t s) {
  KWork w;
  carve(workspace, n_nodes, &w);
  KState init{};
  init.maxiter = maxiter;
  CPFEM_CUDA_TRY(cudaMemcpyAsync(w.st, &init, sizeof(KState), cudaMemcpyHostToDevice, s));
  if (precond != 0) {
    k_precond_setup<TRANS><<<(unsigned)ceil_div(n_nodes, 128), 128, 0, s>>>(n_nodes, nrp, ncol, vals, precond, w.minv);
    CPFEM_CUDA_TRY(cudaGetLastError());
  }
  const unsigned sb = (unsigned)std::min<int64_t>(kSpmvBlocks, ceil_div(n_nodes, kSpmvThreads / 32));
  const unsigned vb = (unsigned)std::min<int64_t>(kVecBlocks, ceil_div(n_nodes, kVecThreads));
  k_bicg_init<TRANS><<<sb, kSpmvThreads, 0, s>>>(n_nodes, nrp, ncol, ntpos, vals, b, x, w, tol, atol);
  CPFEM_CUDA_TRY(cudaGetLastError());
  int done = 0;
  int launched = 0;
  const int chunk = std::max(1, check_every);
  while (launched < maxiter) {
    const int n_it = std::min(chunk, maxiter - launched);
    for (int it = 0; it < n_it; ++it) {
      k_bicg_p<<<vb, kVecThreads, 0, s>>>(n_nodes, w, precond);
      k_bicg_q<TRANS><<<sb, kSpmvThreads, 0, s>>>(n_nodes, nrp, ncol, ntpos, vals, w);
      k_bicg_s<<<vb, kVecThreads, 0, s>>>(n_nodes, w, precond);
      k_bicg_t<TRANS><<<sb, kSpmvThreads, 0, s>>>(n_nodes, nrp, ncol, ntpos, vals, w);
      k_bicg_x<<<vb, kVecThreads, 0, s>>>(n_nodes, w, x);
    }
    CPFEM_CUDA_TRY(cudaGetLastError());
    launched += n_it;
    CPFEM_CUDA_TRY(cudaMemcpyAsync(&done, &w.st->done, sizeof(int), cudaMemcpyDeviceToHost, s));
    CPFEM_CUDA_TRY(cudaStreamSynchronize(s));
    if (done) break;
  }
  KState fin;
  CPFEM_CUDA_TRY(cudaMemcpyAsync(&fin, w.st, sizeof(KState), cudaMemcpyDeviceToHost, s));
  CPFEM_CUDA_TRY(cudaStreamSynchronize(s));
  info[0] = fin.k;
  info[1] = (fin.rs <= fin.atol2) ? 1 : 0;
  return CPFEM_OK;
}

}  // namespace cpfem

using namespace cpfem;

extern "C" {

int cpfem_spmv(int32_t num_nodes, const int32_t* node_rowptr, const int32_t* node_cols, const double* values,
               const double* x, double* y, void* stream) {
  if (num_nodes == 0) return CPFEM_OK;
  CPFEM_REQUIRE(num_nodes > 0 && node_rowptr && node_cols && values && x && y, "bad spmv arguments");
  const unsigned sb = (unsigned)std::min<int64_t>(kSpmvBlocks, ceil_div(num_nodes, kSpmvThreads / 32));
  k_spmv<false><<<sb, kSpmvThreads, 0, (cudaStream_t)stream>>>(num_nodes, node_rowptr, node_cols, nullptr, values,
                                                               x, y);
  CPFEM_CUDA_TRY(cudaGetLastError());
  return CPFEM_OK;
}

int cpfem_spmv_t(int32_t num_nodes, const int32_t* node_rowptr, const int32_t* node_cols,
                 const int32_t* node_tpos, const double* values, const double* x, double* y, void* stream) {
  if (num_nodes == 0) return CPFEM_OK;
  CPFEM_REQUIRE(num_nodes > 0 && node_rowptr && node_cols && node_tpos && values && x && y,
                "bad spmv_t arguments");
  const unsigned sb = (unsigned)std::min<int64_t>(kSpmvBlocks, ceil_div(num_nodes, kSpmvThreads / 32));
  k_spmv<true><<<sb, kSpmvThreads, 0, (cudaStream_t)stream>>>(num_nodes, node_rowptr, node_cols, node_tpos,
                                                              values, x, y);
  CPFEM_CUDA_TRY(cudaGetLastError());
  return CPFEM_OK;
}

size_t cpfem_bicgstab_workspace_bytes(int32_t num_nodes) { return carve(nullptr, num_nodes, nullptr); }

int cpfem_bicgstab(int32_t num_nodes, const int32_t* node_rowptr, const int32_t* node_cols,
                   const int32_t* node_tpos, const double* values, const double* b, double* x,
                   int32_t precond, int32_t transpose, double tol, double atol, int32_t maxiter,
                   int32_t check_every, void* workspace, int32_t* info, void* stream) {
  CPFEM_REQUIRE(info != nullptr, "info is null");
  info[0] = 0;
  info[1] = 1;
  if (num_nodes == 0) return CPFEM_OK;
  CPFEM_REQUIRE(num_nodes > 0 && node_rowptr && node_cols && values && b && x && workspace,
                "bad bicgstab arguments");
  CPFEM_REQUIRE(((uintptr_t)workspace & 255) == 0, "workspace must be 256-byte aligned");
  CPFEM_REQUIRE(precond >= 0 && precond <= 2, "precond must be 0, 1 or 2");
  CPFEM_REQUIRE(maxiter >= 0, "maxiter must be >= 0");
  CPFEM_REQUIRE(!transpose || node_tpos != nullptr, "transpose needs node_tpos");
  cudaStream_t s = (cudaStream_t)stream;
  if (transpose)
    return run_bicgstab<true>(num_nodes, node_rowptr, node_cols, node_tpos, values, b, x, precond, tol, atol,
                              maxiter, check_every, workspace, info, s);
  return run_bicgstab<false>(num_nodes, node_rowptr, node_cols, nullptr, values, b, x, precond, tol, atol,
                             maxiter, check_every, workspace, info, s);
}

}  // extern "C"
