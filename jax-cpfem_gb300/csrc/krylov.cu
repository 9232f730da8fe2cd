// Sliced-ELL SpMV and the persistent BiCGSTAB of the cpfem_gb300 C ABI.
//
// Values are stored per group of 32 consecutive nodes (one warp), slot-major, so the
// thread of node a reads its 3x3 blocks with fully coalesced loads and accumulates its
// three rows without any cross-lane reduction -- on GB300 the FP64 pipe, not HBM, is
// the SpMV's limit, and a shuffle reduction would cost as many FP64 adds as the FMAs.
//
// BiCGSTAB runs as one cooperative launch: every block owns a fixed set of nodes, the
// five global dependencies of an iteration (the halo of phat and shat, four dot
// products) are crossed with a grid barrier, and every block reduces the per-block
// partial sums in the same fixed order, so all blocks hold bitwise-identical scalars
// and take the same branch.  Barrier waits are bounded: a block that waits too long sets
// an error flag and the solve returns CPFEM_ERR_SOLVE.
#include <algorithm>
#include <string>

#include "cpfem_common.cuh"
#include "reduce.cuh"

namespace cpfem {

constexpr int kPThreads = 256;
constexpr int kMaxBlocks = 2048;
constexpr long long kSpinLimit = 1LL << 25;   // ~1-3 s of polling at ~50 ns per poll

struct GridSync {
  unsigned int count;
  unsigned int gen;
  int error;
  int pad;
};

struct SolveOut {
  int k;
  int error;
  double rs;
  double atol2;
};

struct KWork {
  GridSync* sync;
  SolveOut* out;
  double* partials;   // 2 buffers x 4 values x kMaxBlocks
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
  tmp.sync = (GridSync*)take(sizeof(GridSync));
  tmp.out = (SolveOut*)take(sizeof(SolveOut));
  tmp.partials = (double*)take(sizeof(double) * 2 * 4 * kMaxBlocks);
  double** vecs[] = {&tmp.r, &tmp.rhat, &tmp.p, &tmp.q, &tmp.s, &tmp.t, &tmp.phat, &tmp.shat};
  for (double** v : vecs) *v = (double*)take(sizeof(double) * n);
  tmp.minv = (double*)take(sizeof(double) * 9 * n_nodes);
  if (w) *w = tmp;
  return off;
}

// Three rows of node a of A x (or A^T x).  COHERENT selects L2 loads for x, needed when
// x was written by other blocks earlier in the same launch.
template <bool TRANS, bool COHERENT>
__device__ __forceinline__ void sell_rows(const cpfem_sell_t& L, const double* __restrict__ vals,
                                          const double* x, int64_t a, double* acc) {
  const int64_t g = a >> 5;
  const int lane = (int)(a & 31);
  const int64_t c0 = L.group_off[g] + lane;
  const double* v0 = vals + 9 * L.group_off[g] + lane;
  const int w = L.group_width[g];
  double a0 = 0.0, a1 = 0.0, a2 = 0.0;
#pragma unroll 3
  for (int j = 0; j < w; ++j) {
    const int64_t b = __ldg(&L.cols[c0 + 32 * j]);
    double x0, x1, x2;
    if (COHERENT) {
      x0 = __ldcg(&x[3 * b]); x1 = __ldcg(&x[3 * b + 1]); x2 = __ldcg(&x[3 * b + 2]);
    } else {
      x0 = __ldg(&x[3 * b]); x1 = __ldg(&x[3 * b + 1]); x2 = __ldg(&x[3 * b + 2]);
    }
    if (!TRANS) {
      const double* vj = v0 + 288 * j;
      a0 = fma(__ldg(&vj[0]), x0, fma(__ldg(&vj[32]), x1, fma(__ldg(&vj[64]), x2, a0)));
      a1 = fma(__ldg(&vj[96]), x0, fma(__ldg(&vj[128]), x1, fma(__ldg(&vj[160]), x2, a1)));
      a2 = fma(__ldg(&vj[192]), x0, fma(__ldg(&vj[224]), x1, fma(__ldg(&vj[256]), x2, a2)));
    } else {
      // A^T[3a+i][3b+k] = A[3b+k][3a+i]: node b, slot tpos, row k, column i
      const int64_t tp = __ldg(&L.tpos[c0 + 32 * j]);
      const double* vb = vals + 9 * L.group_off[b >> 5] + (b & 31) + 288 * tp;
      a0 = fma(__ldg(&vb[0]), x0, fma(__ldg(&vb[96]), x1, fma(__ldg(&vb[192]), x2, a0)));
      a1 = fma(__ldg(&vb[32]), x0, fma(__ldg(&vb[128]), x1, fma(__ldg(&vb[224]), x2, a1)));
      a2 = fma(__ldg(&vb[64]), x0, fma(__ldg(&vb[160]), x1, fma(__ldg(&vb[256]), x2, a2)));
    }
  }
  acc[0] = a0;
  acc[1] = a1;
  acc[2] = a2;
}

template <bool TRANS>
__global__ void __launch_bounds__(256) k_spmv(const cpfem_sell_t L, const double* __restrict__ vals,
                                              const double* __restrict__ x, double* __restrict__ y) {
  for (int64_t a = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; a < L.num_nodes;
       a += (int64_t)gridDim.x * blockDim.x) {
    double acc[3];
    sell_rows<TRANS, false>(L, vals, x, a, acc);
    y[3 * a] = acc[0];
    y[3 * a + 1] = acc[1];
    y[3 * a + 2] = acc[2];
  }
}

// Diagonal (precond 1) or inverted 3x3 diagonal block (precond 2) per node.
template <bool TRANS>
__global__ void k_precond_setup(const cpfem_sell_t L, const double* __restrict__ vals, int precond,
                                double* __restrict__ minv) {
  const int64_t a = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= L.num_nodes) return;
  const double* v0 = vals + 9 * L.group_off[a >> 5] + (a & 31) + 288 * (int64_t)L.diag_slot[a];
  double blk[9];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const double v = v0[32 * (3 * i + k)];
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

// Sense-counting grid barrier for a cooperative launch, with a bounded wait.
__device__ __forceinline__ bool grid_barrier(GridSync* gs, unsigned int& gen) {
  __shared__ int s_ok;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned int my = gen;
    int ok = 1;
    const unsigned int arrived = atomicAdd(&gs->count, 1u);
    if (arrived == gridDim.x - 1) {
      atomicExch(&gs->count, 0u);
      __threadfence();
      atomicExch(&gs->gen, my + 1u);
    } else {
      volatile unsigned int* vg = &gs->gen;
      long long spins = 0;
      while (*vg == my) {
        if (++spins > kSpinLimit) {
          ok = 0;
          atomicExch(&gs->error, 1);
          break;
        }
        __nanosleep(32);
      }
    }
    __threadfence();
    s_ok = ok && (*(volatile int*)&gs->error == 0);
  }
  __syncthreads();
  gen += 1u;
  return s_ok != 0;
}

// Publish this block's NV partial sums, cross the grid barrier, and reduce all blocks'
// partials in a fixed order (the same in every block).  Returns false on barrier error.
template <int NV>
__device__ __forceinline__ bool grid_reduce(double (&v)[NV], double* partials, GridSync* gs, unsigned int& gen,
                                            double* smem, double* bcast) {
  block_sum<NV>(v, smem);
  if (threadIdx.x == 0)
#pragma unroll
    for (int k = 0; k < NV; ++k) partials[k * gridDim.x + blockIdx.x] = v[k];
  const bool ok = grid_barrier(gs, gen);
  if (threadIdx.x < 32) {
    double acc[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k) acc[k] = 0.0;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += 32)
#pragma unroll
      for (int k = 0; k < NV; ++k) acc[k] += __ldcg(&partials[k * gridDim.x + b]);
    warp_sum<NV>(acc);
    if (threadIdx.x == 0)
#pragma unroll
      for (int k = 0; k < NV; ++k) bcast[k] = acc[k];
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < NV; ++k) v[k] = bcast[k];
  __syncthreads();
  return ok;
}

template <bool TRANS>
__global__ void __launch_bounds__(kPThreads) k_bicgstab(const cpfem_sell_t L, const double* __restrict__ vals,
                                                        const double* __restrict__ b, double* __restrict__ x,
                                                        KWork w, int precond, double tol, double atol,
                                                        int maxiter) {
  __shared__ double smem[4 * 32];
  __shared__ double bcast[4];
  const int64_t n = L.num_nodes;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t t0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  unsigned int gen = 0u;
  int buf = 0;
  auto parts = [&]() {
    double* p = w.partials + (size_t)buf * 4 * kMaxBlocks;
    buf ^= 1;
    return p;
  };
  bool ok = true;

  // r = b - A x0 ; rhat = p = q = r
  double v2[2] = {0.0, 0.0};
  for (int64_t a = t0; a < n; a += stride) {
    double acc[3];
    sell_rows<TRANS, true>(L, vals, x, a, acc);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      const int64_t d = 3 * a + i;
      const double bv = b[d];
      const double rv = bv - acc[i];
      w.r[d] = rv; w.rhat[d] = rv; w.p[d] = rv; w.q[d] = rv;
      v2[0] = fma(bv, bv, v2[0]);
      v2[1] = fma(rv, rv, v2[1]);
    }
  }
  ok = grid_reduce<2>(v2, parts(), w.sync, gen, smem, bcast) && ok;
  const double atol2 = fmax(tol * tol * v2[0], atol * atol);
  double rs = v2[1], rho_new = v2[1], rho = 1.0, alpha = 1.0, omega = 1.0;
  int k = 0;

  while (ok && rs > atol2 && k < maxiter && k >= 0) {
    const double beta = rho_new / rho * alpha / omega;
    // p = r + beta (p - omega q); phat = M p
    for (int64_t a = t0; a < n; a += stride) {
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
    ok = grid_barrier(w.sync, gen) && ok;
    // q = A phat ; alpha = rho_new / (rhat . q)
    double v1[1] = {0.0};
    for (int64_t a = t0; a < n; a += stride) {
      double acc[3];
      sell_rows<TRANS, true>(L, vals, w.phat, a, acc);
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        const int64_t d = 3 * a + i;
        w.q[d] = acc[i];
        v1[0] = fma(w.rhat[d], acc[i], v1[0]);
      }
    }
    ok = grid_reduce<1>(v1, parts(), w.sync, gen, smem, bcast) && ok;
    alpha = rho_new / v1[0];
    // s = r - alpha q ; shat = M s ; exit_early = s.s < atol2
    double vs[1] = {0.0};
    for (int64_t a = t0; a < n; a += stride) {
      double sv[3], sh[3];
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        const int64_t d = 3 * a + i;
        sv[i] = w.r[d] - alpha * w.q[d];
        w.s[d] = sv[i];
        vs[0] = fma(sv[i], sv[i], vs[0]);
      }
      apply_m(precond, w.minv, a, sv, sh);
#pragma unroll
      for (int i = 0; i < 3; ++i) w.shat[3 * a + i] = sh[i];
    }
    ok = grid_reduce<1>(vs, parts(), w.sync, gen, smem, bcast) && ok;
    const bool early = vs[0] < atol2;
    // t = A shat ; omega = (t.s)/(t.t)
    double vt[2] = {0.0, 0.0};
    for (int64_t a = t0; a < n; a += stride) {
      double acc[3];
      sell_rows<TRANS, true>(L, vals, w.shat, a, acc);
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        const int64_t d = 3 * a + i;
        w.t[d] = acc[i];
        vt[0] = fma(acc[i], w.s[d], vt[0]);
        vt[1] = fma(acc[i], acc[i], vt[1]);
      }
    }
    ok = grid_reduce<2>(vt, parts(), w.sync, gen, smem, bcast) && ok;
    omega = vt[0] / vt[1];
    // x and r update
    double vr[2] = {0.0, 0.0};
    for (int64_t a = t0; a < n; a += stride) {
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        const int64_t d = 3 * a + i;
        double rv;
        if (early) {
          x[d] = x[d] + alpha * w.phat[d];
          rv = w.s[d];
        } else {
          x[d] = x[d] + (alpha * w.phat[d] + omega * w.shat[d]);
          rv = w.s[d] - omega * w.t[d];
        }
        w.r[d] = rv;
        vr[0] = fma(rv, rv, vr[0]);
        vr[1] = fma(w.rhat[d], rv, vr[1]);
      }
    }
    ok = grid_reduce<2>(vr, parts(), w.sync, gen, smem, bcast) && ok;
    int kn = (omega == 0.0 || alpha == 0.0) ? -11 : k + 1;
    if (rho_new == 0.0) kn = -10;
    k = kn;
    rho = rho_new;
    rho_new = vr[1];
    rs = vr[0];
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    w.out->k = k;
    w.out->error = ok ? 0 : 1;
    w.out->rs = rs;
    w.out->atol2 = atol2;
  }
}

static int sm_count_and_blocks(const void* fn, int* blocks_per_sm, int* sms) {
  int dev = 0;
  CPFEM_CUDA_TRY(cudaGetDevice(&dev));
  CPFEM_CUDA_TRY(cudaDeviceGetAttribute(sms, cudaDevAttrMultiProcessorCount, dev));
  CPFEM_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, fn, kPThreads, 0));
  return CPFEM_OK;
}

template <bool TRANS>
static int run_bicgstab(const cpfem_sell_t& L, const double* vals, const double* b, double* x, int precond,
                        double tol, double atol, int32_t maxiter, void* workspace, int32_t* info, cudaStream_t s) {
  KWork w;
  carve(workspace, L.num_nodes, &w);
  CPFEM_CUDA_TRY(cudaMemsetAsync(w.sync, 0, sizeof(GridSync), s));
  if (precond != 0) {
    k_precond_setup<TRANS><<<(unsigned)ceil_div(L.num_nodes, 128), 128, 0, s>>>(L, vals, precond, w.minv);
    CPFEM_CUDA_TRY(cudaGetLastError());
  }
  int per_sm = 0, sms = 0;
  int rc = sm_count_and_blocks((const void*)k_bicgstab<TRANS>, &per_sm, &sms);
  if (rc) return rc;
  if (per_sm < 1) {
    set_error("persistent BiCGSTAB kernel cannot be resident");
    return CPFEM_ERR_CUDA;
  }
  int64_t blocks = std::min<int64_t>((int64_t)per_sm * sms, ceil_div(L.num_nodes, kPThreads));
  blocks = std::max<int64_t>(1, std::min<int64_t>(blocks, kMaxBlocks));
  cpfem_sell_t Lc = L;
  const double* bb = b;
  double* xx = x;
  int pc = precond;
  double tl = tol, at = atol;
  int mi = maxiter;
  void* args[] = {&Lc, &vals, &bb, &xx, &w, &pc, &tl, &at, &mi};
  CPFEM_CUDA_TRY(cudaLaunchCooperativeKernel((const void*)k_bicgstab<TRANS>, dim3((unsigned)blocks),
                                             dim3(kPThreads), args, 0, s));
  SolveOut out;
  CPFEM_CUDA_TRY(cudaMemcpyAsync(&out, w.out, sizeof(SolveOut), cudaMemcpyDeviceToHost, s));
  CPFEM_CUDA_TRY(cudaStreamSynchronize(s));
  info[0] = out.k;
  info[1] = (out.rs <= out.atol2) ? 1 : 0;
  if (out.error) {
    set_error("BiCGSTAB grid barrier timed out");
    return CPFEM_ERR_SOLVE;
  }
  return CPFEM_OK;
}

static bool sell_ok(const cpfem_sell_t* L) {
  return L && L->num_nodes >= 0 && L->group_off && L->group_width && L->cols && L->diag_slot &&
         L->num_groups == (L->num_nodes + 31) / 32;
}

}  // namespace cpfem

using namespace cpfem;

extern "C" {

int cpfem_spmv(const cpfem_sell_t* sell, const double* values, const double* x, double* y, int32_t transpose,
               void* stream) {
  CPFEM_REQUIRE(sell_ok(sell) && values && x && y, "bad spmv arguments");
  CPFEM_REQUIRE(!transpose || sell->tpos, "transpose needs tpos");
  if (sell->num_nodes == 0) return CPFEM_OK;
  const unsigned blocks = (unsigned)std::min<int64_t>(ceil_div(sell->num_nodes, 256), 8 * 152);
  if (transpose)
    k_spmv<true><<<blocks, 256, 0, (cudaStream_t)stream>>>(*sell, values, x, y);
  else
    k_spmv<false><<<blocks, 256, 0, (cudaStream_t)stream>>>(*sell, values, x, y);
  CPFEM_CUDA_TRY(cudaGetLastError());
  return CPFEM_OK;
}

size_t cpfem_bicgstab_workspace_bytes(int32_t num_nodes) { return carve(nullptr, num_nodes, nullptr); }

int cpfem_bicgstab(const cpfem_sell_t* sell, const double* values, const double* b, double* x, int32_t precond,
                   int32_t transpose, double tol, double atol, int32_t maxiter, void* workspace, int32_t* info,
                   void* stream) {
  CPFEM_REQUIRE(info != nullptr, "info is null");
  info[0] = 0;
  info[1] = 1;
  CPFEM_REQUIRE(sell_ok(sell), "bad layout");
  if (sell->num_nodes == 0) return CPFEM_OK;
  CPFEM_REQUIRE(values && b && x && workspace, "bad bicgstab arguments");
  CPFEM_REQUIRE(((uintptr_t)workspace & 255) == 0, "workspace must be 256-byte aligned");
  CPFEM_REQUIRE(precond >= 0 && precond <= 2, "precond must be 0, 1 or 2");
  CPFEM_REQUIRE(maxiter >= 0, "maxiter must be >= 0");
  CPFEM_REQUIRE(!transpose || sell->tpos != nullptr, "transpose needs tpos");
  cudaStream_t s = (cudaStream_t)stream;
  if (transpose) return run_bicgstab<true>(*sell, values, b, x, precond, tol, atol, maxiter, workspace, info, s);
  return run_bicgstab<false>(*sell, values, b, x, precond, tol, atol, maxiter, workspace, info, s);
}

}  // extern "C"

// ---- batched BiCGSTAB: one CTA per instance, ragged instances from a work queue ------
namespace cpfem {

constexpr int kBThreads = 1024;

struct BWork {
  double *r, *rhat, *p, *q, *s, *t, *phat, *shat, *minv;
  unsigned int* queue;   // next entry of the active list
};

static size_t carve_batched(void* base, int64_t n_nodes, BWork* w) {
  const int64_t n = 3 * n_nodes;
  char* p = (char*)base;
  size_t off = 0;
  auto take = [&](size_t bytes) {
    char* q = p ? p + off : nullptr;
    off += align256(bytes);
    return q;
  };
  BWork tmp;
  tmp.queue = (unsigned int*)take(sizeof(unsigned int));
  double** vecs[] = {&tmp.r, &tmp.rhat, &tmp.p, &tmp.q, &tmp.s, &tmp.t, &tmp.phat, &tmp.shat};
  for (double** v : vecs) *v = (double*)take(sizeof(double) * n);
  tmp.minv = (double*)take(sizeof(double) * 9 * n_nodes);
  if (w) *w = tmp;
  return off;
}

template <int NV>
__device__ __forceinline__ void cta_sum(double (&v)[NV], double* smem) {
  block_sum<NV>(v, smem);
  __shared__ double bc[4];
  if (threadIdx.x == 0)
#pragma unroll
    for (int k = 0; k < NV; ++k) bc[k] = v[k];
  __syncthreads();
#pragma unroll
  for (int k = 0; k < NV; ++k) v[k] = bc[k];
  __syncthreads();
}

// Each CTA takes instances from the queue; instance `inst` owns nodes
// [node_off[inst], node_off[inst+1]).  Threads walk the instance's nodes group-aligned so
// a warp reads one sliced-ELL group.
__global__ void __launch_bounds__(kBThreads) k_bicgstab_batched(
    const cpfem_sell_t L, const double* __restrict__ vals, const double* __restrict__ b, double* __restrict__ x,
    BWork w, int precond, double tol, double atol, int maxiter, int n_active, const int32_t* __restrict__ active,
    const int32_t* __restrict__ node_off, int32_t* __restrict__ info) {
  __shared__ double smem[4 * 32];
  __shared__ int s_job;
  for (;;) {
    if (threadIdx.x == 0) s_job = (int)atomicAdd(w.queue, 1u);
    __syncthreads();
    const int job = s_job;
    __syncthreads();
    if (job >= n_active) break;
    const int inst = active[job];
    const int64_t n0 = node_off[inst], n1 = node_off[inst + 1];
    const int64_t a0 = (n0 >> 5) << 5;
    // r = b - A x0 ; rhat = p = q = r
    double v2[2] = {0.0, 0.0};
    for (int64_t a = a0 + threadIdx.x; a < n1; a += blockDim.x) {
      if (a < n0) continue;
      double acc[3];
      sell_rows<false, true>(L, vals, x, a, acc);
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        const int64_t d = 3 * a + i;
        const double bv = b[d];
        const double rv = bv - acc[i];
        w.r[d] = rv; w.rhat[d] = rv; w.p[d] = rv; w.q[d] = rv;
        v2[0] = fma(bv, bv, v2[0]);
        v2[1] = fma(rv, rv, v2[1]);
      }
    }
    cta_sum<2>(v2, smem);
    const double atol2 = fmax(tol * tol * v2[0], atol * atol);
    double rs = v2[1], rho_new = v2[1], rho = 1.0, alpha = 1.0, omega = 1.0;
    int k = 0;
    while (rs > atol2 && k < maxiter && k >= 0) {
      const double beta = rho_new / rho * alpha / omega;
      for (int64_t a = a0 + threadIdx.x; a < n1; a += blockDim.x) {
        if (a < n0) continue;
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
      __syncthreads();
      double v1[1] = {0.0};
      for (int64_t a = a0 + threadIdx.x; a < n1; a += blockDim.x) {
        if (a < n0) continue;
        double acc[3];
        sell_rows<false, true>(L, vals, w.phat, a, acc);
#pragma unroll
        for (int i = 0; i < 3; ++i) {
          const int64_t d = 3 * a + i;
          w.q[d] = acc[i];
          v1[0] = fma(w.rhat[d], acc[i], v1[0]);
        }
      }
      cta_sum<1>(v1, smem);
      alpha = rho_new / v1[0];
      double vs[1] = {0.0};
      for (int64_t a = a0 + threadIdx.x; a < n1; a += blockDim.x) {
        if (a < n0) continue;
        double sv[3], sh[3];
#pragma unroll
        for (int i = 0; i < 3; ++i) {
          const int64_t d = 3 * a + i;
          sv[i] = w.r[d] - alpha * w.q[d];
          w.s[d] = sv[i];
          vs[0] = fma(sv[i], sv[i], vs[0]);
        }
        apply_m(precond, w.minv, a, sv, sh);
#pragma unroll
        for (int i = 0; i < 3; ++i) w.shat[3 * a + i] = sh[i];
      }
      cta_sum<1>(vs, smem);
      const bool early = vs[0] < atol2;
      double vt[2] = {0.0, 0.0};
      for (int64_t a = a0 + threadIdx.x; a < n1; a += blockDim.x) {
        if (a < n0) continue;
        double acc[3];
        sell_rows<false, true>(L, vals, w.shat, a, acc);
#pragma unroll
        for (int i = 0; i < 3; ++i) {
          const int64_t d = 3 * a + i;
          w.t[d] = acc[i];
          vt[0] = fma(acc[i], w.s[d], vt[0]);
          vt[1] = fma(acc[i], acc[i], vt[1]);
        }
      }
      cta_sum<2>(vt, smem);
      omega = vt[0] / vt[1];
      double vr[2] = {0.0, 0.0};
      for (int64_t a = a0 + threadIdx.x; a < n1; a += blockDim.x) {
        if (a < n0) continue;
#pragma unroll
        for (int i = 0; i < 3; ++i) {
          const int64_t d = 3 * a + i;
          double rv;
          if (early) {
            x[d] = x[d] + alpha * w.phat[d];
            rv = w.s[d];
          } else {
            x[d] = x[d] + (alpha * w.phat[d] + omega * w.shat[d]);
            rv = w.s[d] - omega * w.t[d];
          }
          w.r[d] = rv;
          vr[0] = fma(rv, rv, vr[0]);
          vr[1] = fma(w.rhat[d], rv, vr[1]);
        }
      }
      cta_sum<2>(vr, smem);
      int kn = (omega == 0.0 || alpha == 0.0) ? -11 : k + 1;
      if (rho_new == 0.0) kn = -10;
      k = kn;
      rho = rho_new;
      rho_new = vr[1];
      rs = vr[0];
    }
    if (threadIdx.x == 0) {
      info[2 * inst] = k;
      info[2 * inst + 1] = (rs <= atol2) ? 1 : 0;
    }
    __syncthreads();
  }
}

}  // namespace cpfem

extern "C" {

size_t cpfem_bicgstab_batched_workspace_bytes(int32_t num_nodes) {
  return cpfem::carve_batched(nullptr, num_nodes, nullptr);
}

int cpfem_bicgstab_batched(const cpfem_sell_t* sell, const double* values, const double* b, double* x,
                           int32_t precond, double tol, double atol, int32_t maxiter, int32_t num_active,
                           const int32_t* active, const int32_t* node_off, void* workspace, int32_t* info,
                           void* stream) {
  using namespace cpfem;
  CPFEM_REQUIRE(sell_ok(sell), "bad layout");
  if (num_active == 0 || sell->num_nodes == 0) return CPFEM_OK;
  CPFEM_REQUIRE(values && b && x && active && node_off && workspace && info, "bad batched bicgstab arguments");
  CPFEM_REQUIRE(((uintptr_t)workspace & 255) == 0, "workspace must be 256-byte aligned");
  CPFEM_REQUIRE(precond >= 0 && precond <= 2 && maxiter >= 0 && num_active > 0, "bad solver settings");
  cudaStream_t s = (cudaStream_t)stream;
  BWork w;
  carve_batched(workspace, sell->num_nodes, &w);
  CPFEM_CUDA_TRY(cudaMemsetAsync(w.queue, 0, sizeof(unsigned int), s));
  if (precond != 0) {
    k_precond_setup<false><<<(unsigned)ceil_div(sell->num_nodes, 128), 128, 0, s>>>(*sell, values, precond, w.minv);
    CPFEM_CUDA_TRY(cudaGetLastError());
  }
  int dev = 0, sms = 0;
  CPFEM_CUDA_TRY(cudaGetDevice(&dev));
  CPFEM_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const unsigned blocks = (unsigned)std::min<int64_t>(num_active, (int64_t)sms);
  k_bicgstab_batched<<<blocks, kBThreads, 0, s>>>(*sell, values, b, x, w, precond, tol, atol, maxiter, num_active,
                                                 active, node_off, info);
  CPFEM_CUDA_TRY(cudaGetLastError());
  return CPFEM_OK;
}

}  // extern "C"

// ---- allocation-free variant ---------------------------------------------------------
// Some callers cannot allocate device memory at all: a host code that owns every device
// byte through its own pool, or a caller that must not grow its footprint inside a
// real-time loop.  cpfem_bicgstab_noalloc gives them the same solver with its scratch
// (Krylov vectors, preconditioner, reduction partials, barrier words) in a fixed
// file-scope device array, sized for CPFEM_NOALLOC_MAX_NODES nodes.  The array lives in
// every GPU that loads the library until the process exits.
#include <mutex>

namespace cpfem {

constexpr int64_t kNoAllocMaxNodes = CPFEM_NOALLOC_MAX_NODES;

static size_t noalloc_bytes_needed() { return carve(nullptr, kNoAllocMaxNodes, nullptr); }

// 256-byte aligned scratch; its size is fixed at compile time from the carve layout of
// kNoAllocMaxNodes nodes (checked again at run time).
static __device__ __align__(256) unsigned char g_noalloc_scratch[CPFEM_NOALLOC_SCRATCH_BYTES];

static std::mutex g_noalloc_mutex;
static void* g_noalloc_ptr[256] = {nullptr};

// Device address of the scratch on the current device.  Host code must not use the
// symbol's name as an address: it is a host-side stand-in.  Resolved once per device.
static int noalloc_scratch(void** out) {
  int dev = 0;
  CPFEM_CUDA_TRY(cudaGetDevice(&dev));
  CPFEM_REQUIRE(dev >= 0 && dev < 256, "device index out of range");
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (g_noalloc_ptr[dev] == nullptr) {
    void* ptr = nullptr;
    CPFEM_CUDA_TRY(cudaGetSymbolAddress(&ptr, g_noalloc_scratch));
    CPFEM_REQUIRE(ptr != nullptr && ((uintptr_t)ptr & 255) == 0, "scratch address is not 256-byte aligned");
    g_noalloc_ptr[dev] = ptr;
  }
  *out = g_noalloc_ptr[dev];
  return CPFEM_OK;
}

}  // namespace cpfem

extern "C" int cpfem_bicgstab_noalloc(const cpfem_sell_t* sell, const double* values, const double* b, double* x,
                                      int32_t precond, int32_t transpose, double tol, double atol,
                                      int32_t maxiter, int32_t* info, void* stream) {
  using namespace cpfem;
  CPFEM_REQUIRE(info != nullptr, "info is null");
  info[0] = 0;
  info[1] = 1;
  CPFEM_REQUIRE(sell_ok(sell), "bad layout");
  if (sell->num_nodes > kNoAllocMaxNodes) {
    set_error("cpfem_bicgstab_noalloc: " + std::to_string(sell->num_nodes) + " nodes exceed the fixed scratch of " +
              std::to_string((long long)kNoAllocMaxNodes) + " nodes; use cpfem_bicgstab with a caller workspace");
    return CPFEM_ERR_SIZE;
  }
  CPFEM_REQUIRE(noalloc_bytes_needed() <= sizeof(g_noalloc_scratch), "scratch smaller than its layout");
  void* ws = nullptr;
  int rc = noalloc_scratch(&ws);
  if (rc != CPFEM_OK) return rc;
  // run_bicgstab clears the barrier words and writes every vector before reading it
  return cpfem_bicgstab(sell, values, b, x, precond, transpose, tol, atol, maxiter, ws, info, stream);
}
