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
#include <cmath>
#include <cstring>
#include <type_traits>
#include <vector>
#include <string>

#include "cpfem_common.cuh"
#include "reduce.cuh"

namespace cpfem {

constexpr int kPThreads = 256;
constexpr int kMaxBlocks = 2048;
constexpr long long kSpinLimit = 1LL << 25;   // ~1-3 s of polling at ~50 ns per poll

struct GridSync {
  unsigned int count;   // arrivals so far (monotonic within a launch)
  unsigned int gen;     // unused (kept for the layout)
  int error;
  int pad;
};

// the launch's report, written by the kernel into the workspace (the public layout)
using SolveOut = cpfem_solve_report_t;
static_assert(sizeof(SolveOut) == 72 && offsetof(SolveOut, true_rs) == 56, "solve report layout");

// cpfem_krylov_opts_t.flags: also form the true residual of the returned x; report
// asynchronously instead of waiting for the solve
constexpr int kKrylovTrueResidual = 1;
constexpr int kKrylovDeferred = 2;

static thread_local SolveOut g_last_solve = {0, 0, 0.0, 0.0, 0.0, 0.0, 0.0, 0, 0, -1.0, 0.0};

struct KWork {
  GridSync* sync;
  SolveOut* out;
  double* partials;   // 2 buffers x 4 values x kMaxBlocks
  double *r, *rhat, *p, *q, *s, *t, *phat, *shat, *minv;
};

static constexpr size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

// Bytes carve() lays out for n_nodes nodes, as a compile-time expression (the fixed scratch
// of the allocation-free entry point is checked against it when the library is built).
static constexpr size_t carve_bytes(int64_t n_nodes) {
  return align256(sizeof(GridSync)) + align256(sizeof(SolveOut)) + align256(sizeof(double) * 2 * 4 * kMaxBlocks) +
         8 * align256(sizeof(double) * 3 * (size_t)n_nodes) + align256(sizeof(double) * 9 * (size_t)n_nodes);
}

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

__device__ __forceinline__ double mad(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ float mad(float a, float b, float c) { return fmaf(a, b, c); }

// An operator value in the precision R of the product.  FP64 -> FP32 by integer operations on
// the two words of the double (exponent re-bias, mantissa truncated to 23 bits, magnitudes
// below FP32's normal range flushed to zero), so the FP32 V-cycle can read the resident FP64
// operator without a conversion instruction per value on GB300's narrow FP64 pipe.  The
// truncation error (< 2^-23 relative) is below what an FP32 preconditioner resolves.
template <typename R>
__device__ __forceinline__ R opval(double v);
template <>
__device__ __forceinline__ double opval<double>(double v) { return v; }
template <>
__device__ __forceinline__ float opval<float>(double v) {
  const unsigned hi = (unsigned)__double2hiint(v), lo = (unsigned)__double2loint(v);
  const int e = (int)((hi >> 20) & 0x7FFu) - 1023 + 127;
  const unsigned bits = (e <= 0) ? (hi & 0x80000000u)
                                 : ((hi & 0x80000000u) | ((unsigned)e << 23) | ((hi & 0xFFFFFu) << 3) | (lo >> 29));
  return __uint_as_float(bits);
}
template <typename R>
__device__ __forceinline__ R opval(float v) { return (R)v; }

// Three rows of node a of A x (or A^T x), in the precision R of the values and x (FP64 for
// the Krylov iteration, FP32 inside a single-precision V-cycle).  COHERENT selects L2
// loads for x, needed when x was written by other blocks earlier in the same launch.
template <bool TRANS, bool COHERENT, typename R, typename VT = R>
__device__ __forceinline__ void sell_rows(const cpfem_sell_t& L, const VT* __restrict__ vals,
                                          const R* x, int64_t a, R* acc) {
  const int64_t g = a >> 5;
  const int lane = (int)(a & 31);
  const int64_t c0 = L.group_off[g] + lane;
  const VT* v0 = vals + 9 * L.group_off[g] + lane;
  const int w = L.group_width[g];
  // two accumulators per row (even / odd slots): six independent FMA chains keep the FP64
  // pipe fed at one thread per node
  R e0 = R(0), e1 = R(0), e2 = R(0), o0 = R(0), o1 = R(0), o2 = R(0);
  auto slot = [&](int j, R& a0, R& a1, R& a2) {
    const int64_t b = __ldg(&L.cols[c0 + 32 * j]);
    R x0, x1, x2;
    if (COHERENT) {
      x0 = __ldcg(&x[3 * b]); x1 = __ldcg(&x[3 * b + 1]); x2 = __ldcg(&x[3 * b + 2]);
    } else {
      x0 = __ldg(&x[3 * b]); x1 = __ldg(&x[3 * b + 1]); x2 = __ldg(&x[3 * b + 2]);
    }
    if (!TRANS) {
      const VT* vj = v0 + 288 * j;
      a0 = mad(opval<R>(__ldg(&vj[0])), x0, mad(opval<R>(__ldg(&vj[32])), x1, mad(opval<R>(__ldg(&vj[64])), x2, a0)));
      a1 = mad(opval<R>(__ldg(&vj[96])), x0, mad(opval<R>(__ldg(&vj[128])), x1, mad(opval<R>(__ldg(&vj[160])), x2, a1)));
      a2 = mad(opval<R>(__ldg(&vj[192])), x0, mad(opval<R>(__ldg(&vj[224])), x1, mad(opval<R>(__ldg(&vj[256])), x2, a2)));
    } else {
      // A^T[3a+i][3b+k] = A[3b+k][3a+i]: node b, slot tpos, row k, column i
      const int64_t tp = __ldg(&L.tpos[c0 + 32 * j]);
      const VT* vb = vals + 9 * L.group_off[b >> 5] + (b & 31) + 288 * tp;
      a0 = mad(opval<R>(__ldg(&vb[0])), x0, mad(opval<R>(__ldg(&vb[96])), x1, mad(opval<R>(__ldg(&vb[192])), x2, a0)));
      a1 = mad(opval<R>(__ldg(&vb[32])), x0, mad(opval<R>(__ldg(&vb[128])), x1, mad(opval<R>(__ldg(&vb[224])), x2, a1)));
      a2 = mad(opval<R>(__ldg(&vb[64])), x0, mad(opval<R>(__ldg(&vb[160])), x1, mad(opval<R>(__ldg(&vb[256])), x2, a2)));
    }
  };
  int j = 0;
#pragma unroll 2
  for (; j + 1 < w; j += 2) {
    slot(j, e0, e1, e2);
    slot(j + 1, o0, o1, o2);
  }
  if (j < w) slot(j, e0, e1, e2);
  acc[0] = e0 + o0;
  acc[1] = e1 + o1;
  acc[2] = e2 + o2;
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

__device__ __forceinline__ unsigned int ld_acquire_u32(const unsigned int* p) {
  unsigned int v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void red_release_add_u32(unsigned int* p, unsigned int v) {
  asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Barrier over the nb blocks that share gs (the whole grid of a cooperative launch, or a
// team of it).  gs->count only grows (it is zeroed before the launch): the k-th barrier is
// complete when it reaches k*nb.  Thread 0 arrives with a release reduction, which
// publishes every write the block made before the __syncthreads, and waits with acquire
// loads; no reset is needed, so the last arrival costs no extra round trip.  The wait is
// bounded: after kSpinLimit polls the block records an error (also in *gerr) and returns
// false instead of hanging.
__device__ __forceinline__ bool counted_barrier(GridSync* gs, unsigned int nb, unsigned int& gen, int* gerr) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned int target = (gen + 1u) * nb;
    int ok = 1;
    red_release_add_u32(&gs->count, 1u);
    long long spins = 0;
    while (ld_acquire_u32(&gs->count) < target) {
      if (++spins > kSpinLimit) {
        ok = 0;
        atomicExch(&gs->error, 1);
        if (gerr != nullptr) atomicExch(gerr, 1);
        break;
      }
      if (spins > 32) __nanosleep(32);
    }
    s_ok = ok && (*(volatile int*)&gs->error == 0);
  }
  __syncthreads();
  gen += 1u;
  return s_ok != 0;
}

__device__ __forceinline__ bool grid_barrier(GridSync* gs, unsigned int& gen) {
  return counted_barrier(gs, gridDim.x, gen, nullptr);
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

// ---- geometric multigrid (precond 3) ------------------------------------------------
// Levels of a structured box of nodes, x fastest.  Fine node i of level l and coarse node
// I of level l+1 are linked when i is within one fine node of 2I in every direction, with
// the trilinear weight prod_d (1 if i_d = 2 I_d else 1/2).

__device__ __forceinline__ void mg_xyz(int64_t a, const int32_t* dims, int& x, int& y, int& z) {
  // node counts fit 32 bits (cpfem_sell_t.num_nodes is int32): 32-bit divisions
  const unsigned ua = (unsigned)a, d0 = (unsigned)dims[0], d1 = (unsigned)dims[1];
  const unsigned q = ua / d0;
  x = (int)(ua - q * d0);
  z = (int)(q / d1);
  y = (int)(q - (unsigned)z * d1);
}

// z = D^-1 v with the stored inverse diagonal block; TRANS uses its transpose, which is
// the inverse of the diagonal block of A^T.
template <bool TRANS, typename R>
__device__ __forceinline__ void mg_apply_minv(const R* __restrict__ minv, int64_t a, const R* v, R* out) {
  const R* bi = minv + 9 * a;
  if (TRANS) {
#pragma unroll
    for (int i = 0; i < 3; ++i) out[i] = mad(bi[i], v[0], mad(bi[3 + i], v[1], bi[6 + i] * v[2]));
  } else {
#pragma unroll
    for (int i = 0; i < 3; ++i) out[i] = mad(bi[3 * i], v[0], mad(bi[3 * i + 1], v[1], bi[3 * i + 2] * v[2]));
  }
}

// One damped block-Jacobi sweep at node a of level 0: T = X + omega Minv (B - A X) (A^T
// when TRANS); B is the Krylov vector being preconditioned (FP64), the rest in precision R.
template <bool TRANS, typename R, typename VT>
__device__ __forceinline__ void mg_sweep(const cpfem_sell_t& S, const VT* V, const R* minv, const double* B,
                                         const R* X, R* T, R omega, int64_t a) {
  R acc[3], r[3], z[3];
  sell_rows<TRANS, true, R, VT>(S, V, X, a, acc);
#pragma unroll
  for (int i = 0; i < 3; ++i) r[i] = (R)B[3 * a + i] - acc[i];
  mg_apply_minv<TRANS>(minv, a, r, z);
#pragma unroll
  for (int i = 0; i < 3; ++i) T[3 * a + i] = mad(omega, z[i], __ldcg(&X[3 * a + i]));
}

// Rows of node a of A x (A^T x when TRANS) restricted to the slots j = q (mod 4) (one
// lane of a quad).
// A vector element written earlier in the launch: an L2 load from global memory (other
// blocks may have written it), a plain load from shared memory (SH).
template <bool SH, typename R>
__device__ __forceinline__ R ldv(const R* p) {
  if constexpr (SH) return *p;
  else return __ldcg(p);
}

// A value of a level operator: read-only for the whole launch, so through the read-only
// cache from global memory, or a plain load from shared memory (SH).
template <bool SH, typename R>
__device__ __forceinline__ R ldc(const R* p) {
  if constexpr (SH) return *p;
  else return __ldg(p);
}

template <bool TRANS, bool SH, typename R, bool SHV = false>
__device__ __forceinline__ void sell_rows_quad(const cpfem_sell_t& L, const R* __restrict__ vals, const R* x,
                                               int64_t a, int q, R* acc) {
  const int64_t g = a >> 5;
  const int lane = (int)(a & 31);
  const int64_t c0 = L.group_off[g] + lane;
  const R* v0 = vals + 9 * L.group_off[g] + lane;
  const int w = L.group_width[g];
  R a0 = R(0), a1 = R(0), a2 = R(0);
#pragma unroll 2
  for (int j = q; j < w; j += 4) {
    const int64_t b = __ldg(&L.cols[c0 + 32 * j]);
    const R x0 = ldv<SH>(&x[3 * b]), x1 = ldv<SH>(&x[3 * b + 1]), x2 = ldv<SH>(&x[3 * b + 2]);
    if (!TRANS) {
      const R* vb = v0 + 288 * j;
      a0 = mad(ldc<SHV>(&vb[0]), x0, mad(ldc<SHV>(&vb[32]), x1, mad(ldc<SHV>(&vb[64]), x2, a0)));
      a1 = mad(ldc<SHV>(&vb[96]), x0, mad(ldc<SHV>(&vb[128]), x1, mad(ldc<SHV>(&vb[160]), x2, a1)));
      a2 = mad(ldc<SHV>(&vb[192]), x0, mad(ldc<SHV>(&vb[224]), x1, mad(ldc<SHV>(&vb[256]), x2, a2)));
    } else {
      const int64_t tp = __ldg(&L.tpos[c0 + 32 * j]);
      const R* vb = vals + 9 * L.group_off[b >> 5] + (b & 31) + 288 * tp;
      a0 = mad(ldc<SHV>(&vb[0]), x0, mad(ldc<SHV>(&vb[96]), x1, mad(ldc<SHV>(&vb[192]), x2, a0)));
      a1 = mad(ldc<SHV>(&vb[32]), x0, mad(ldc<SHV>(&vb[128]), x1, mad(ldc<SHV>(&vb[224]), x2, a1)));
      a2 = mad(ldc<SHV>(&vb[64]), x0, mad(ldc<SHV>(&vb[160]), x1, mad(ldc<SHV>(&vb[256]), x2, a2)));
    }
  }
  acc[0] = a0;
  acc[1] = a1;
  acc[2] = a2;
}

constexpr int kMgMaxWidth = 27;                 // neighbour slots of a structured-box node

// Staged (shared-memory) copies of a block-local level are skewed: the four lanes of a
// node's quad read four consecutive slots, whose sliced-ELL rows (288 values, or 32 index
// entries) start in the same bank, so every slot row is followed by 8 unused words.  Lanes
// (node k, slot phase q) of a warp then read bank k + 8q: no bank conflicts.
constexpr int64_t kStSkew = 8;
__host__ __device__ constexpr int64_t st_val_index(int64_t i) { return i + kStSkew * (i / 288); }
__host__ __device__ constexpr int64_t st_idx_index(int64_t i) { return i + kStSkew * (i >> 5); }
constexpr int64_t kStValRow = 288 + kStSkew, kStIdxRow = 32 + kStSkew;

// sell_rows_quad on a level staged in shared memory: values, x and the index tables
// (group offsets, widths, columns, transposed slots as int32, mg_stage) all there, the
// values and the column / transposed-slot tables in the skewed order above (group offsets
// are multiples of 32 slots, so a group's rows start at a whole skewed row).
template <bool TRANS, typename R>
__device__ __forceinline__ void sell_rows_quad_st(const int* ix, int ng, const R* vals, const R* x, int64_t a,
                                                  int q, R* acc) {
  const int* goff = ix;
  const int* gw = ix + ng + 1;
  const int* cols = gw + ng;
  const int* tpos = cols + kStIdxRow * kMgMaxWidth * ng;
  const int g = (int)(a >> 5);
  const int lane = (int)(a & 31);
  const int gs = goff[g];
  const int c0 = gs + (int)kStSkew * (gs >> 5) + lane;               // st_idx_index(gs + lane)
  const R* v0 = vals + 9 * gs + (int)kStSkew * (gs >> 5) + lane;     // st_val_index(9 gs + lane)
  const int w = gw[g];
  R a0 = R(0), a1 = R(0), a2 = R(0);
#pragma unroll 2
  for (int j = q; j < w; j += 4) {
    const int b = cols[c0 + (int)kStIdxRow * j];
    const R x0 = x[3 * b], x1 = x[3 * b + 1], x2 = x[3 * b + 2];
    if (!TRANS) {
      const R* vb = v0 + kStValRow * j;
      a0 = mad(vb[0], x0, mad(vb[32], x1, mad(vb[64], x2, a0)));
      a1 = mad(vb[96], x0, mad(vb[128], x1, mad(vb[160], x2, a1)));
      a2 = mad(vb[192], x0, mad(vb[224], x1, mad(vb[256], x2, a2)));
    } else {
      const int tp = tpos[c0 + (int)kStIdxRow * j];
      const int gb = goff[b >> 5];
      const R* vb = vals + 9 * gb + (int)kStSkew * (gb >> 5) + (b & 31) + kStValRow * tp;
      a0 = mad(vb[0], x0, mad(vb[96], x1, mad(vb[192], x2, a0)));
      a1 = mad(vb[32], x0, mad(vb[128], x1, mad(vb[224], x2, a1)));
      a2 = mad(vb[64], x0, mad(vb[160], x1, mad(vb[256], x2, a2)));
    }
  }
  acc[0] = a0;
  acc[1] = a1;
  acc[2] = a2;
}

// The arrays of a V-cycle in precision R: FP64 uses the hierarchy's own operators (level
// 0: the system's values), FP32 the single-precision copies cpfem_mg_setup makes.
template <typename R>
struct MgArrays;
template <>
struct MgArrays<double> {
  const cpfem_mg_t& m;
  const double* v0;
  __device__ __forceinline__ const double* values(int l) const { return l == 0 ? v0 : m.values[l]; }
  __device__ __forceinline__ const double* minv(int l) const { return m.minv[l]; }
  __device__ __forceinline__ double* x(int l) const { return m.x[l]; }
  __device__ __forceinline__ double* t(int l) const { return m.t[l]; }
  __device__ __forceinline__ double* r(int l) const { return m.r[l]; }
  __device__ __forceinline__ double* b(int l) const { return m.b[l]; }
};
template <>
struct MgArrays<float> {
  const cpfem_mg_t& m;
  const double* v0;
  __device__ __forceinline__ const float* values(int l) const { return m.values32[l]; }
  __device__ __forceinline__ const float* minv(int l) const { return m.minv32[l]; }
  __device__ __forceinline__ float* x(int l) const { return m.x32[l]; }
  __device__ __forceinline__ float* t(int l) const { return m.t32[l]; }
  __device__ __forceinline__ float* r(int l) const { return m.r32[l]; }
  __device__ __forceinline__ float* b(int l) const { return m.b32[l]; }
};

template <typename R>
__device__ __forceinline__ void quad_sum3(R* v) {
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    v[i] += __shfl_xor_sync(0xffffffffu, v[i], 1);
    v[i] += __shfl_xor_sync(0xffffffffu, v[i], 2);
  }
}

// Level operations of the V-cycle on a coarse level (l >= 1), one quad of lanes per node:
// nodes a = tq, tq + sq, ... (tq = this lane's quad, sq = the quads taking part; a warp
// holds 8 consecutive quads and runs the padded loops in lockstep, so the shuffles always
// see the whole warp); lane 0 of a node's quad owns its writes.  The level's vectors are
// passed explicitly: global arrays on the grid-wide levels, shared memory (SH) on the
// block-local ones.
template <bool TRANS, typename R>
__device__ __forceinline__ void mgq_first_sweep(const cpfem_mg_t& mg, const R* Mi, int l, R* X, const R* B,
                                                int64_t tq, int64_t sq, int q) {
  if (q != 0) return;
  const R om = (R)mg.omega;
  for (int64_t a = tq; a < mg.sell[l].num_nodes; a += sq) {
    R v[3] = {B[3 * a], B[3 * a + 1], B[3 * a + 2]}, z[3];
    mg_apply_minv<TRANS>(Mi, a, v, z);
#pragma unroll
    for (int i = 0; i < 3; ++i) X[3 * a + i] = om * z[i];
  }
}

// T = X + omega Minv (B - A X)  (residual = false)  or  T = B - A X  (residual = true)
template <bool TRANS, bool SH, bool SHV = false, typename R>
__device__ __forceinline__ void mgq_apply(const cpfem_mg_t& mg, const R* V, const R* Mi, int l, const R* X, R* T,
                                          const R* B, bool residual, int64_t tq, int64_t sq, int q,
                                          const int* sidx = nullptr) {
  const cpfem_sell_t& S = mg.sell[l];
  const R om = (R)mg.omega;
  const int64_t n = S.num_nodes, npad = (n + 7) / 8 * 8;
  for (int64_t a = tq; a < npad; a += sq) {
    R acc[3] = {R(0), R(0), R(0)};
    if (a < n) {
      if constexpr (SHV) sell_rows_quad_st<TRANS>(sidx, S.num_groups, V, X, a, q, acc);
      else sell_rows_quad<TRANS, SH, R>(S, V, X, a, q, acc);
    }
    quad_sum3(acc);
    if (a < n && q == 0) {
      R r[3];
#pragma unroll
      for (int i = 0; i < 3; ++i) r[i] = B[3 * a + i] - acc[i];
      if (residual) {
#pragma unroll
        for (int i = 0; i < 3; ++i) T[3 * a + i] = r[i];
      } else {
        R z[3];
        mg_apply_minv<TRANS>(Mi, a, r, z);
#pragma unroll
        for (int i = 0; i < 3; ++i) T[3 * a + i] = mad(om, z[i], X[3 * a + i]);
      }
    }
  }
}

// Bc = P^T Res_l (the level l+1 right-hand side): the 27 fine nodes of a coarse node
// split over its quad.  SH: Res is in shared memory.
template <bool SH, typename R>
__device__ __forceinline__ void mgq_restrict(const cpfem_mg_t& mg, int l, const R* Res, R* Bc, int64_t tq,
                                             int64_t sq, int q) {
  const int32_t* df = mg.dims[l];
  const int32_t* dc = mg.dims[l + 1];
  const int64_t nc = mg.sell[l + 1].num_nodes, ncpad = (nc + 7) / 8 * 8;
  for (int64_t I = tq; I < ncpad; I += sq) {
    R acc[3] = {R(0), R(0), R(0)};
    if (I < nc) {
      int cx, cy, cz;
      mg_xyz(I, dc, cx, cy, cz);
      // the lane's fine neighbours k = q, q+4, ... < 27, unrolled and predicated (an absent
      // neighbour reads node 0 with weight 0), so all their loads are in flight together
#pragma unroll
      for (int kk = 0; kk < 7; ++kk) {
        const int k = q + 4 * kk;
        const int dz = k / 9 - 1, dy = (k / 3) % 3 - 1, dx = k % 3 - 1;
        const int ix = 2 * cx + dx, iy = 2 * cy + dy, iz = 2 * cz + dz;
        const bool in = k < 27 && ix >= 0 && ix < df[0] && iy >= 0 && iy < df[1] && iz >= 0 && iz < df[2];
        const R w = in ? (dx ? R(0.5) : R(1)) * (dy ? R(0.5) : R(1)) * (dz ? R(0.5) : R(1)) : R(0);
        const int64_t i = in ? ix + (int64_t)df[0] * (iy + (int64_t)df[1] * iz) : 0;
#pragma unroll
        for (int c = 0; c < 3; ++c) acc[c] = mad(w, ldv<SH>(&Res[3 * i + c]), acc[c]);
      }
    }
    quad_sum3(acc);
    if (I < nc && q == 0)
#pragma unroll
      for (int c = 0; c < 3; ++c) Bc[3 * I + c] = acc[c];
  }
}

// X_l += P X_{l+1} at the nodes a = first, first + step, ... (masked on Dirichlet dofs of
// level 0).  SH: Xc is in shared memory.
template <bool SH, typename R>
__device__ __forceinline__ void mg_prolong(const cpfem_mg_t& mg, int l, R* X, const R* Xc, int64_t first,
                                           int64_t step) {
  const int32_t* df = mg.dims[l];
  const int32_t* dc = mg.dims[l + 1];
  for (int64_t a = first; a < mg.sell[l].num_nodes; a += step) {
    int ix, iy, iz;
    mg_xyz(a, df, ix, iy, iz);
    const int cx0 = ix >> 1, cy0 = iy >> 1, cz0 = iz >> 1;
    const int nxc = (ix & 1) + 1, nyc = (iy & 1) + 1, nzc = (iz & 1) + 1;
    const R w = ((ix & 1) ? R(0.5) : R(1)) * ((iy & 1) ? R(0.5) : R(1)) * ((iz & 1) ? R(0.5) : R(1));
    R acc[3] = {R(0), R(0), R(0)};
    // the 1, 2, 4 or 8 coarse parents, unrolled over 2x2x2 and predicated (an absent one
    // reads its first parent with weight 0), so all their loads are in flight together
#pragma unroll
    for (int kz = 0; kz < 2; ++kz)
#pragma unroll
      for (int ky = 0; ky < 2; ++ky)
#pragma unroll
        for (int kx = 0; kx < 2; ++kx) {
          const bool in = kx < nxc && ky < nyc && kz < nzc;
          const int64_t I = (cx0 + (in ? kx : 0)) +
                            (int64_t)dc[0] * ((cy0 + (in ? ky : 0)) + (int64_t)dc[1] * (cz0 + (in ? kz : 0)));
          const R wk = in ? w : R(0);
#pragma unroll
          for (int c = 0; c < 3; ++c) acc[c] = mad(wk, ldv<SH>(&Xc[3 * I + c]), acc[c]);
        }
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const bool fixed = (l == 0 && mg.free_dof != nullptr && mg.free_dof[3 * a + c] == 0);
      if (!fixed) X[3 * a + c] += acc[c];
    }
  }
}

constexpr int64_t kMgLocalNodes = 256;   // default: levels this small run inside block 0

// The first block-local level: the coarsest levels, from level 2 on, with at most
// local_nodes nodes (host and device agree on it).
__host__ __device__ inline int mg_first_local(const cpfem_mg_t& mg) {
  const int64_t local_nodes = mg.local_nodes > 0 ? (int64_t)mg.local_nodes : kMgLocalNodes;
  int lb = mg.num_levels;
  for (int l = mg.num_levels - 1; l >= 2 && mg.sell[l].num_nodes <= local_nodes; --l) lb = l;
  return lb;
}

constexpr size_t kMgMaxLocalBytes = 220 * 1024; // shared memory of the block-local levels, at most
constexpr size_t kMgStageBytes = kMgMaxLocalBytes;   // ... also when it holds staged operators

// Shared memory of the block-local levels, in elements of R: x, t, r, b of each level (3
// values per node) and, when everything fits in kMgStageBytes and the V-cycle is FP32, the
// levels' operators (sliced-ELL, at most kMgMaxWidth slots per node) and inverse diagonal
// blocks, staged once per launch.  Host and device derive the same layout.
struct MgShared {
  size_t vec[CPFEM_MG_MAX_LEVELS];
  size_t val[CPFEM_MG_MAX_LEVELS];
  size_t minv[CPFEM_MG_MAX_LEVELS];
  size_t idx[CPFEM_MG_MAX_LEVELS];   // int32: group offsets, group widths, columns, transposed slots
  size_t total;
  bool staged;
};

// int32 entries of a staged level's layout: ng+1 group offsets, ng widths, and the column
// and transposed-slot tables of 32 * kMgMaxWidth slots per group (skewed: kStIdxRow words
// per slot row)
__host__ __device__ inline size_t mg_idx_words(int32_t ng) {
  return 2 * (size_t)ng + 1 + 2 * (size_t)kStIdxRow * (size_t)kMgMaxWidth * ng;
}

__host__ __device__ inline MgShared mg_shared_layout(const cpfem_mg_t& mg, size_t real_bytes) {
  MgShared s{};
  const int lb = mg_first_local(mg);
  size_t off = 0;
  for (int m = lb; m < mg.num_levels; ++m) {
    s.vec[m] = off;
    off += 12 * (size_t)mg.sell[m].num_nodes;
  }
  size_t off_v = off;
  for (int m = lb; m < mg.num_levels; ++m) {
    s.val[m] = off_v;
    off_v += (size_t)kStValRow * (size_t)kMgMaxWidth * (size_t)mg.sell[m].num_groups;
    s.minv[m] = off_v;
    off_v += 9 * (size_t)mg.sell[m].num_nodes;
    s.idx[m] = off_v;   // in 4-byte words, which the staged (FP32) layout's elements are
    off_v += mg_idx_words(mg.sell[m].num_groups);
  }
  s.staged = real_bytes == sizeof(float) && lb < mg.num_levels && off_v * real_bytes <= kMgStageBytes;
  s.total = (s.staged ? off_v : off) * real_bytes;
  return s;
}

extern __shared__ __align__(16) unsigned char mg_shared[];

// Block 0, once per launch: the block-local levels' operators and inverse diagonal blocks
// to shared memory (when the layout stages them).
// Returns whether they were staged (every level within kMgMaxWidth slots per node).
template <typename R>
__device__ bool mg_stage(const cpfem_mg_t& mg, const MgArrays<R>& A, const MgShared& lay) {
  if (!lay.staged) return false;
  for (int m = mg_first_local(mg); m < mg.num_levels; ++m)
    if (mg.sell[m].group_off[mg.sell[m].num_groups] > 32 * (int64_t)kMgMaxWidth * mg.sell[m].num_groups) return false;
  R* sh = reinterpret_cast<R*>(mg_shared);
  for (int m = mg_first_local(mg); m < mg.num_levels; ++m) {
    const cpfem_sell_t& S = mg.sell[m];
    const int64_t nv = 9 * S.group_off[S.num_groups];
    const R* V = A.values(m);
    const R* Mi = A.minv(m);
    for (int64_t i = threadIdx.x; i < nv; i += blockDim.x) sh[lay.val[m] + st_val_index(i)] = V[i];
    for (int64_t i = threadIdx.x; i < 9 * (int64_t)S.num_nodes; i += blockDim.x) sh[lay.minv[m] + i] = Mi[i];
    int* ix = reinterpret_cast<int*>(sh + lay.idx[m]);
    const int ng = S.num_groups;
    const int64_t ns = S.group_off[ng];
    int* cols = ix + 2 * ng + 1;
    int* tpos = cols + kStIdxRow * kMgMaxWidth * ng;
    for (int64_t i = threadIdx.x; i <= ng; i += blockDim.x) ix[i] = (int)S.group_off[i];
    for (int64_t i = threadIdx.x; i < ng; i += blockDim.x) ix[ng + 1 + i] = S.group_width[i];
    for (int64_t i = threadIdx.x; i < ns; i += blockDim.x) {
      cols[st_idx_index(i)] = S.cols[i];
      tpos[st_idx_index(i)] = (S.tpos != nullptr) ? S.tpos[i] : 0;
    }
  }
  __syncthreads();
  return true;
}

// Block 0: the block-local levels lb .. L-1 on its shared memory -- restriction of the
// grid-wide level lb-1's residual, down sweeps, the coarsest level, up sweeps -- and level
// lb's iterate copied to the global array the grid-wide prolongation reads.  SHV: the
// operators were staged (mg_stage); otherwise they are read from global memory.
template <bool TRANS, bool SHV, typename R>
__device__ void mg_local_cycle(const cpfem_mg_t& mg, const MgArrays<R>& A, const MgShared& lay, int lb,
                               const R* Res, const bool* down_t, const bool* up_t, int q) {
  const int L = mg.num_levels;
  const int64_t tqb = threadIdx.x >> 2, sqb = blockDim.x >> 2;   // block-local quads
  R* sh = reinterpret_cast<R*>(mg_shared);
  auto vec = [&](int m, int k) { return sh + lay.vec[m] + (size_t)k * 3 * mg.sell[m].num_nodes; };  // x t r b
  auto V = [&](int m) { return SHV ? (const R*)(sh + lay.val[m]) : A.values(m); };
  auto Mi = [&](int m) { return SHV ? (const R*)(sh + lay.minv[m]) : A.minv(m); };
  auto Ix = [&](int m) { return SHV ? reinterpret_cast<const int*>(sh + lay.idx[m]) : (const int*)nullptr; };
  mgq_restrict<false>(mg, lb - 1, Res, vec(lb, 3), tqb, sqb, q);
  for (int m = lb; m < L; ++m) {
    R* Xm = vec(m, 0);
    R* Tm = vec(m, 1);
    mgq_first_sweep<TRANS>(mg, Mi(m), m, Xm, vec(m, 3), tqb, sqb, q);
    const int nswm = (m == L - 1) ? mg.coarse_sweeps : mg.pre_sweeps;
    for (int k = 1; k < nswm; ++k) {
      __syncthreads();
      mgq_apply<TRANS, true, SHV>(mg, V(m), Mi(m), m, Xm, Tm, vec(m, 3), false, tqb, sqb, q, Ix(m));
      R* tmp = Xm; Xm = Tm; Tm = tmp;
    }
    if (m == L - 1) break;
    __syncthreads();
    mgq_apply<TRANS, true, SHV>(mg, V(m), Mi(m), m, Xm, vec(m, 2), vec(m, 3), true, tqb, sqb, q, Ix(m));
    __syncthreads();
    mgq_restrict<true>(mg, m, vec(m, 2), vec(m + 1, 3), tqb, sqb, q);
  }
  for (int m = L - 2; m >= lb; --m) {
    R* Xm = down_t[m] ? vec(m, 1) : vec(m, 0);
    R* Tm = down_t[m] ? vec(m, 0) : vec(m, 1);
    const R* Xc = (m + 1 == L - 1 ? down_t[m + 1] : up_t[m + 1]) ? vec(m + 1, 1) : vec(m + 1, 0);
    __syncthreads();
    if (q == 0) mg_prolong<true>(mg, m, Xm, Xc, tqb, sqb);
    for (int k = 0; k < mg.post_sweeps; ++k) {
      __syncthreads();
      mgq_apply<TRANS, true, SHV>(mg, V(m), Mi(m), m, Xm, Tm, vec(m, 3), false, tqb, sqb, q, Ix(m));
      R* tmp = Xm; Xm = Tm; Tm = tmp;
    }
  }
  const bool in_t = (lb == L - 1) ? down_t[lb] : up_t[lb];
  const R* src = in_t ? vec(lb, 1) : vec(lb, 0);
  R* dst = in_t ? A.t(lb) : A.x(lb);
  __syncthreads();
  for (int64_t i = threadIdx.x; i < 3 * mg.sell[lb].num_nodes; i += blockDim.x) dst[i] = src[i];
}

// One V-cycle out = M^-1 in over every block of the cooperative launch, in precision R
// (in and out are the FP64 Krylov vectors).  Level 0 uses the caller's one-thread-per-node
// grid-stride mapping (so input written by this thread needs no barrier); coarser levels
// give every node a quad of lanes, so their few nodes still hide load latency.  The levels
// (from level 2 on) with at most local_nodes nodes run inside block 0 on vectors in its
// shared memory (mg_local_cycle), while the other blocks wait at the next grid barrier.
// Which of x / t holds a level's iterate follows from the sweep counts alone, so every
// block knows it.  Returns with out complete for this thread's own nodes.
template <bool TRANS, typename R>
__device__ void mg_vcycle(const cpfem_mg_t& mg, const double* __restrict__ vals0, const double* in, double* out,
                          int64_t t0, int64_t stride, GridSync* gs, unsigned int& gen, bool& ok, bool staged) {
  const MgArrays<R> A{mg, vals0};
  const int L = mg.num_levels;
  const R om = (R)mg.omega;
  const int64_t tq = t0 >> 2, sq = stride >> 2;
  const int q = (int)(t0 & 3);
  const int lb = mg_first_local(mg);                             // first block-local level
  // where each level's iterate lives after its down sweeps / after its up sweeps
  bool down_t[CPFEM_MG_MAX_LEVELS], up_t[CPFEM_MG_MAX_LEVELS];
  for (int l = 0; l < L; ++l) {
    const int nsw = (l == L - 1) ? mg.coarse_sweeps : mg.pre_sweeps;
    down_t[l] = ((nsw - 1) & 1) != 0;
    up_t[l] = (l == L - 1) ? down_t[l] : (down_t[l] != ((mg.post_sweeps & 1) != 0));
  }
  // ---- grid-wide levels 0 .. lb-1, down
  for (int l = 0; l < lb; ++l) {
    const cpfem_sell_t& S = mg.sell[l];
    const R* V = A.values(l);
    const R* Mi = A.minv(l);
    R* X = A.x(l);
    R* T = A.t(l);
    const int64_t n = S.num_nodes;
    if (l == 0) {
      for (int64_t a = t0; a < n; a += stride) {
        R v[3] = {(R)in[3 * a], (R)in[3 * a + 1], (R)in[3 * a + 2]}, z[3];
        mg_apply_minv<TRANS>(Mi, a, v, z);
#pragma unroll
        for (int i = 0; i < 3; ++i) X[3 * a + i] = om * z[i];
      }
    } else {
      mgq_first_sweep<TRANS>(mg, Mi, l, X, A.b(l), tq, sq, q);
    }
    const int nsw = (l == L - 1) ? mg.coarse_sweeps : mg.pre_sweeps;
    for (int k = 1; k < nsw; ++k) {
      ok = grid_barrier(gs, gen) && ok;
      if (l == 0) {
        // level 0 reads the system's FP64 values (no FP32 copy next to them in L2)
        for (int64_t a = t0; a < n; a += stride) mg_sweep<TRANS>(S, vals0, Mi, in, X, T, om, a);
      } else {
        mgq_apply<TRANS, false>(mg, V, Mi, l, X, T, A.b(l), false, tq, sq, q);
      }
      R* tmp = X; X = T; T = tmp;
    }
    if (l == L - 1) break;
    ok = grid_barrier(gs, gen) && ok;
    R* Res = A.r(l);
    if (l == 0) {
      for (int64_t a = t0; a < n; a += stride) {
        R acc[3];
        sell_rows<TRANS, true, R, double>(S, vals0, X, a, acc);
#pragma unroll
        for (int i = 0; i < 3; ++i) {
          const R rv = (R)in[3 * a + i] - acc[i];
          Res[3 * a + i] = (mg.free_dof != nullptr && mg.free_dof[3 * a + i] == 0) ? R(0) : rv;
        }
      }
    } else {
      mgq_apply<TRANS, false>(mg, V, Mi, l, X, Res, A.b(l), true, tq, sq, q);
    }
    ok = grid_barrier(gs, gen) && ok;
    if (l + 1 < lb) {
      mgq_restrict<false>(mg, l, Res, A.b(l + 1), tq, sq, q);
    } else if (blockIdx.x == 0) {
      const MgShared lay = mg_shared_layout(mg, sizeof(R));
      if (staged) mg_local_cycle<TRANS, true>(mg, A, lay, lb, (const R*)Res, down_t, up_t, q);
      else mg_local_cycle<TRANS, false>(mg, A, lay, lb, (const R*)Res, down_t, up_t, q);
    }
  }
  // ---- grid-wide levels lb-1 .. 0, up
  for (int l = lb - 1; l >= 0; --l) {
    if (l == L - 1) continue;
    const cpfem_sell_t& S = mg.sell[l];
    const R* V = A.values(l);
    const R* Mi = A.minv(l);
    R* X = down_t[l] ? A.t(l) : A.x(l);
    R* T = down_t[l] ? A.x(l) : A.t(l);
    const R* Xc = (l + 1 == L - 1 ? down_t[l + 1] : up_t[l + 1]) ? A.t(l + 1) : A.x(l + 1);
    ok = grid_barrier(gs, gen) && ok;
    if (l == 0) mg_prolong<false>(mg, 0, X, Xc, t0, stride);
    else if (q == 0) mg_prolong<false>(mg, l, X, Xc, tq, sq);
    for (int k = 0; k < mg.post_sweeps; ++k) {
      ok = grid_barrier(gs, gen) && ok;
      if (l == 0) {
        for (int64_t a = t0; a < S.num_nodes; a += stride) mg_sweep<TRANS>(S, vals0, Mi, in, X, T, om, a);
      } else {
        mgq_apply<TRANS, false>(mg, V, Mi, l, X, T, A.b(l), false, tq, sq, q);
      }
      R* tmp = X; X = T; T = tmp;
    }
  }
  const R* X0 = up_t[0] ? A.t(0) : A.x(0);
  for (int64_t a = t0; a < mg.sell[0].num_nodes; a += stride)
#pragma unroll
    for (int i = 0; i < 3; ++i) out[3 * a + i] = (double)X0[3 * a + i];
}

// MGP: 0 the point preconditioners of precond 0..2, 1 the FP64 V-cycle, 2 the FP32 V-cycle.
// The FP32 V-cycle runs one block per SM (every block reserves the shared memory of the
// block-local levels), so it may take the whole register file: with up to 255 registers
// the fine-level row products keep more loads in flight (219.8 vs 237.4 us per iteration at
// 32^3, measured per phase).
template <bool TRANS, int MGP>
__global__ void __launch_bounds__(kPThreads, MGP == 2 ? 1 : 3) k_bicgstab(const cpfem_sell_t L, const double* __restrict__ vals,
                                                        const double* __restrict__ b, double* __restrict__ x,
                                                        KWork w, int precond, double tol, double atol,
                                                        int maxiter, int max_restarts, const cpfem_mg_t mg) {
  constexpr bool MG = MGP != 0;
  using MgReal = typename std::conditional<MGP == 2, float, double>::type;
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
  bool staged = false;
  if constexpr (MG) {
    // block 0 keeps the block-local levels' operators in shared memory for the whole solve
    if (blockIdx.x == 0) staged = mg_stage<MgReal>(mg, MgArrays<MgReal>{mg, vals}, mg_shared_layout(mg, sizeof(MgReal)));
  }

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
  if (blockIdx.x == 0 && threadIdx.x == 0) w.out->bb = v2[0];   // b.b, written now: nothing stays live
  const double rs0 = fmax(v2[1], atol2);
  double rs = v2[1], rho_new = v2[1], rho = 1.0, alpha = 1.0, omega = 1.0;
  int k = 0, restarts = 0;

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
      if constexpr (!MG) {
        apply_m(precond, w.minv, a, pv, ph);
#pragma unroll
        for (int i = 0; i < 3; ++i) w.phat[3 * a + i] = ph[i];
      }
    }
    if constexpr (MG) mg_vcycle<TRANS, MgReal>(mg, vals, w.p, w.phat, t0, stride, w.sync, gen, ok, staged);
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
      if constexpr (!MG) {
        apply_m(precond, w.minv, a, sv, sh);
#pragma unroll
        for (int i = 0; i < 3; ++i) w.shat[3 * a + i] = sh[i];
      }
    }
    if constexpr (!MG) {
      ok = grid_reduce<1>(vs, parts(), w.sync, gen, smem, bcast) && ok;   // also the shat halo barrier
    } else {
      // the V-cycle starts on this thread's own s; s.s joins the t reduction below
      mg_vcycle<TRANS, MgReal>(mg, vals, w.s, w.shat, t0, stride, w.sync, gen, ok, staged);
      ok = grid_barrier(w.sync, gen) && ok;
    }
    // t = A shat ; omega = (t.s)/(t.t)
    double vt[3] = {0.0, 0.0, MG ? vs[0] : 0.0};
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
    if constexpr (MG) {
      ok = grid_reduce<3>(vt, parts(), w.sync, gen, smem, bcast) && ok;
      vs[0] = vt[2];
    } else {
      double vt2[2] = {vt[0], vt[1]};
      ok = grid_reduce<2>(vt2, parts(), w.sync, gen, smem, bcast) && ok;
      vt[0] = vt2[0];
      vt[1] = vt2[1];
    }
    const bool early = vs[0] < atol2;
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
    rho = rho_new;
    rho_new = vr[1];
    rs = vr[0];
    // an FP32 V-cycle cannot resolve the near-null modes of a near-singular system (its
    // rounding, amplified by the condition number, swamps them); a residual that grew by
    // 1e8 or went non-finite ends the solve with -12 so the caller can re-solve in FP64
    if (MGP == 2 && !(rs <= 1e16 * rs0)) kn = -12;
    if (kn < 0 && kn != -12 && restarts < max_restarts && ok && rs > atol2) {
      // restart at the current x: rhat = p = q = r = b - A x (x is complete: the last
      // reduction crossed the grid barrier after every block wrote its part)
      ++restarts;
      double v3[1] = {0.0};
      for (int64_t a = t0; a < n; a += stride) {
        double acc[3];
        sell_rows<TRANS, true>(L, vals, x, a, acc);
#pragma unroll
        for (int i = 0; i < 3; ++i) {
          const int64_t d = 3 * a + i;
          const double rv = b[d] - acc[i];
          w.r[d] = rv; w.rhat[d] = rv; w.p[d] = rv; w.q[d] = rv;
          v3[0] = fma(rv, rv, v3[0]);
        }
      }
      ok = grid_reduce<1>(v3, parts(), w.sync, gen, smem, bcast) && ok;
      rs = v3[0];
      rho_new = v3[0];
      rho = alpha = omega = 1.0;
      k = k + 1;
    } else {
      k = kn;
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    w.out->true_rs = -1.0;
    w.out->restarts = restarts;
    w.out->k = k;
    w.out->error = ok ? 0 : 1;
    w.out->rs = rs;
    w.out->atol2 = atol2;
    w.out->rho = rho;
    w.out->alpha = alpha;
    w.out->omega = omega;
  }
}

// ||b - A x||^2 in block partials (fixed grid, fixed order inside a block).
template <bool TRANS>
__global__ void __launch_bounds__(kVecThreads) k_true_residual(const cpfem_sell_t L, const double* __restrict__ vals,
                                                               const double* __restrict__ b,
                                                               const double* __restrict__ x, double* partials) {
  __shared__ double smem[4 * 32];
  double v[1] = {0.0};
  for (int64_t a = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; a < L.num_nodes;
       a += (int64_t)gridDim.x * blockDim.x) {
    double acc[3];
    sell_rows<TRANS, false>(L, vals, x, a, acc);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      const double r = b[3 * a + i] - acc[i];
      v[0] = fma(r, r, v[0]);
    }
  }
  block_sum<1>(v, smem);
  if (threadIdx.x == 0) partials[blockIdx.x] = v[0];
}

__global__ void k_sum_partials(const double* __restrict__ partials, int n, double* out) {
  double v[1] = {0.0};
  for (int i = threadIdx.x; i < n; i += 32) v[0] += partials[i];
  warp_sum<1>(v);
  if (threadIdx.x == 0) *out = v[0];
}

static int sm_count_and_blocks(const void* fn, int* blocks_per_sm, int* sms, size_t dyn_smem = 0) {
  int dev = 0;
  CPFEM_CUDA_TRY(cudaGetDevice(&dev));
  CPFEM_CUDA_TRY(cudaDeviceGetAttribute(sms, cudaDevAttrMultiProcessorCount, dev));
  CPFEM_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, fn, kPThreads, dyn_smem));
  return CPFEM_OK;
}


template <bool TRANS>
static int run_bicgstab(const cpfem_sell_t& L, const double* vals, const double* b, double* x, int precond,
                        double tol, double atol, int32_t maxiter, void* workspace, int32_t* info, cudaStream_t s,
                        int max_restarts = 0, const cpfem_mg_t* mgp = nullptr, int grid_blocks = 0,
                        int flags = 0, cpfem_solve_report_t* report = nullptr) {
  KWork w;
  carve(workspace, L.num_nodes, &w);
  CPFEM_CUDA_TRY(cudaMemsetAsync(w.sync, 0, sizeof(GridSync), s));
  if (precond == 1 || precond == 2) {
    k_precond_setup<TRANS><<<(unsigned)ceil_div(L.num_nodes, 128), 128, 0, s>>>(L, vals, precond, w.minv);
    CPFEM_CUDA_TRY(cudaGetLastError());
  }
  cpfem_mg_t mg;
  memset(&mg, 0, sizeof(mg));
  if (precond == 3) mg = *mgp;
  int per_sm = 0, sms = 0;
  const void* kfn = (precond != 3)      ? (const void*)k_bicgstab<TRANS, 0>
                    : (mg.precision == 1) ? (const void*)k_bicgstab<TRANS, 2>
                                          : (const void*)k_bicgstab<TRANS, 1>;
  size_t dyn = 0;
  if (precond == 3) {
    dyn = mg_shared_layout(mg, mg.precision == 1 ? sizeof(float) : sizeof(double)).total;
    if (dyn > kMgMaxLocalBytes) {
      set_error("multigrid local_nodes too large: the block-local levels do not fit in shared memory");
      return CPFEM_ERR_ARG;
    }
    if (dyn > 48 * 1024) CPFEM_CUDA_TRY(cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn));
  }
  int rc = sm_count_and_blocks(kfn, &per_sm, &sms, dyn);
  if (rc) return rc;
  if (per_sm < 1) {
    set_error("persistent BiCGSTAB kernel cannot be resident");
    return CPFEM_ERR_CUDA;
  }
  int64_t blocks = std::min<int64_t>((int64_t)per_sm * sms, ceil_div(L.num_nodes, kPThreads));
  if (grid_blocks > 0) blocks = std::min<int64_t>((int64_t)per_sm * sms, grid_blocks);
  blocks = std::max<int64_t>(1, std::min<int64_t>(blocks, kMaxBlocks));
  cpfem_sell_t Lc = L;
  const double* bb = b;
  double* xx = x;
  int pc = precond;
  double tl = tol, at = atol;
  int mi = maxiter, mr = max_restarts;
  void* args[] = {&Lc, &vals, &bb, &xx, &w, &pc, &tl, &at, &mi, &mr, &mg};
  CPFEM_CUDA_TRY(cudaLaunchCooperativeKernel(kfn, dim3((unsigned)blocks), dim3(kPThreads), args, dyn, s));
  if (flags & kKrylovTrueResidual) {
    // ||b - A x||^2 of the returned x: block partials, then one block sums them in order
    // (deterministic), into the SolveOut read below -- no extra synchronisation
    k_true_residual<TRANS><<<kVecBlocks, kVecThreads, 0, s>>>(L, vals, b, x, w.partials);
    CPFEM_CUDA_TRY(cudaGetLastError());
    k_sum_partials<<<1, 32, 0, s>>>(w.partials, kVecBlocks, &w.out->true_rs);
    CPFEM_CUDA_TRY(cudaGetLastError());
  }
  if (flags & kKrylovDeferred) {
    // queued behind the solve and the true residual: the caller reads it after its next
    // synchronisation of the stream
    CPFEM_CUDA_TRY(cudaMemcpyAsync(report, w.out, sizeof(SolveOut), cudaMemcpyDeviceToHost, s));
    return CPFEM_OK;
  }
  SolveOut out;
  CPFEM_CUDA_TRY(cudaMemcpyAsync(&out, w.out, sizeof(SolveOut), cudaMemcpyDeviceToHost, s));
  CPFEM_CUDA_TRY(cudaStreamSynchronize(s));
  info[0] = out.k;
  info[1] = (out.rs <= out.atol2) ? 1 : 0;
  g_last_solve = out;
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

static int mg_check(const cpfem_mg_t* mg, const cpfem_sell_t* sell) {
  CPFEM_REQUIRE(mg != nullptr, "precond 3 needs a multigrid hierarchy (opts.mg)");
  const int L = mg->num_levels;
  CPFEM_REQUIRE(L >= 2 && L <= CPFEM_MG_MAX_LEVELS, "multigrid num_levels must be 2..CPFEM_MG_MAX_LEVELS");
  CPFEM_REQUIRE(mg->pre_sweeps >= 1 && mg->post_sweeps >= 0 && mg->coarse_sweeps >= 1, "bad multigrid sweep counts");
  CPFEM_REQUIRE(mg->omega > 0.0 && mg->omega < 2.0, "multigrid omega must lie in (0, 2)");
  CPFEM_REQUIRE(sell == nullptr || mg->sell[0].num_nodes == sell->num_nodes, "level 0 must be the system's layout");
  CPFEM_REQUIRE(mg->precision == 0 || mg->precision == 1, "multigrid precision must be 0 (FP64) or 1 (FP32)");
  CPFEM_REQUIRE(mg->local_nodes >= 0, "multigrid local_nodes must be >= 0");
  const bool single = mg->precision == 1;
  for (int l = 0; l < L; ++l) {
    const int64_t n = (int64_t)mg->dims[l][0] * mg->dims[l][1] * mg->dims[l][2];
    CPFEM_REQUIRE(mg->dims[l][0] >= 1 && mg->dims[l][1] >= 1 && mg->dims[l][2] >= 1 && n == mg->sell[l].num_nodes,
                  "multigrid dims do not match the level's node count");
    CPFEM_REQUIRE(sell_ok(&mg->sell[l]) && mg->minv[l], "multigrid level arrays missing");
    CPFEM_REQUIRE(single ? ((l == 0 || mg->values32[l]) && mg->minv32[l] && mg->x32[l] && mg->t32[l])
                         : (mg->x[l] && mg->t[l]),
                  "multigrid work arrays missing");
    CPFEM_REQUIRE(mg->slot[l], "multigrid slot table missing");
    if (l + 1 < L) {
      CPFEM_REQUIRE(single ? mg->r32[l] != nullptr : mg->r[l] != nullptr, "multigrid residual array missing");
      const int64_t need = (int64_t)((mg->dims[l][0] - 1) / 2 + 1) * mg->dims[l][1] * mg->dims[l][2];
      CPFEM_REQUIRE(mg->scratch[0] && mg->scratch[1] && mg->scratch_nodes >= need,
                    "multigrid scratch missing or too small");
    }
    if (l >= 1) {
      CPFEM_REQUIRE(mg->values[l] && (single ? mg->b32[l] != nullptr : mg->b[l] != nullptr),
                    "multigrid coarse arrays missing");
      for (int d = 0; d < 3; ++d)
        CPFEM_REQUIRE((mg->dims[l - 1][d] - 1) % 2 == 0 && mg->dims[l][d] == (mg->dims[l - 1][d] - 1) / 2 + 1,
                      "each multigrid level must halve the cell counts of the finer one");
    }
  }
  return CPFEM_OK;
}

// Galerkin coarse operator P^T A P by three 1-D passes: P = P_z (x) P_y (x) P_x, so
// coarsening one direction at a time keeps a 27-point stencil and needs 7 (same coarse
// neighbour) or 3 (next one) fine pairs per output block instead of up to 343.  One thread
// per (output node, stencil offset); input and output stencils are [node][27][9]; the
// first pass reads the sliced-ELL fine operator through its slot table (Dirichlet dofs of
// level 0 left out on both sides), the last writes the coarse sliced-ELL operator.
// Fixed summation order: reproducible.
__global__ void __launch_bounds__(256) k_mg_rap_dir(int dir, int ix, int iy, int iz, int ox, int oy, int oz,
                                                    const cpfem_sell_t F, const double* __restrict__ vf,
                                                    const int8_t* __restrict__ slot_in,
                                                    const double* __restrict__ sin_,
                                                    const int8_t* __restrict__ free_dof, double* __restrict__ sout,
                                                    const cpfem_sell_t C, const int8_t* __restrict__ slot_out,
                                                    double* __restrict__ vc) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t nout = (int64_t)ox * oy * oz;
  if (t >= 27 * nout) return;
  const int64_t o = t / 27;
  const int off = (int)(t % 27);
  int oc[3] = {(int)(o % ox), (int)((o / ox) % oy), (int)(o / ((int64_t)ox * oy))};
  int d[3] = {off % 3 - 1, (off / 3) % 3 - 1, off / 9 - 1};
  const int din[3] = {ix, iy, iz};
  const int del = d[dir];
  double acc[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) acc[k] = 0.0;
  for (int a = -1; a <= 1; ++a)
    for (int b = -1; b <= 1; ++b) {
      const int e = 2 * del + b - a;      // input offset along dir
      if (e < -1 || e > 1) continue;
      int ic[3] = {oc[0], oc[1], oc[2]};
      ic[dir] = 2 * oc[dir] + a;
      int jc[3] = {ic[0] + d[0], ic[1] + d[1], ic[2] + d[2]};
      jc[dir] = ic[dir] + e;
      bool inside = true;
#pragma unroll
      for (int k = 0; k < 3; ++k)
        inside = inside && ic[k] >= 0 && ic[k] < din[k] && jc[k] >= 0 && jc[k] < din[k];
      if (!inside) continue;
      const int64_t i = ic[0] + (int64_t)ix * (ic[1] + (int64_t)iy * ic[2]);
      int ed[3] = {d[0], d[1], d[2]};
      ed[dir] = e;
      const int code = (ed[2] + 1) * 9 + (ed[1] + 1) * 3 + (ed[0] + 1);
      const double w = (a ? 0.5 : 1.0) * (b ? 0.5 : 1.0);
      if (sin_ == nullptr) {
        const int sf = slot_in[27 * i + code];
        if (sf < 0) continue;
        const int64_t j = jc[0] + (int64_t)ix * (jc[1] + (int64_t)iy * jc[2]);
        const double* blk = vf + 9 * F.group_off[i >> 5] + (i & 31) + 288LL * sf;
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            if (free_dof != nullptr && (free_dof[3 * i + r] == 0 || free_dof[3 * j + c] == 0)) continue;
            acc[3 * r + c] = fma(w, __ldg(&blk[32 * (3 * r + c)]), acc[3 * r + c]);
          }
      } else {
        const double* blk = sin_ + 9 * (27 * i + code);
#pragma unroll
        for (int k = 0; k < 9; ++k) acc[k] = fma(w, __ldg(&blk[k]), acc[k]);
      }
    }
  if (sout != nullptr) {
#pragma unroll
    for (int k = 0; k < 9; ++k) sout[9 * (27 * o + off) + k] = acc[k];
  } else {
    const int s = slot_out[27 * o + off];
    if (s < 0) return;
    double* blk = vc + 9 * C.group_off[o >> 5] + (o & 31) + 288LL * s;
#pragma unroll
    for (int k = 0; k < 9; ++k) blk[32 * k] = acc[k];
  }
}

// FP32 copy of n values, or of a sliced-ELL value array (9 * group_off[num_groups] values,
// read on the device) when slots != nullptr.
__global__ void __launch_bounds__(256) k_to_f32(const double* __restrict__ in, float* __restrict__ out, int64_t n,
                                                const int64_t* __restrict__ slots) {
  const int64_t m = slots != nullptr ? 9 * slots[0] : n;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = (float)in[i];
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

int cpfem_mg_setup(const cpfem_mg_t* mg, const double* values0, void* stream) {
  CPFEM_REQUIRE(values0 != nullptr, "values0 is null");
  int rc = mg_check(mg, nullptr);
  if (rc != CPFEM_OK) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  k_precond_setup<false><<<(unsigned)ceil_div(mg->sell[0].num_nodes, 128), 128, 0, s>>>(mg->sell[0], values0, 2,
                                                                                         mg->minv[0]);
  CPFEM_CUDA_TRY(cudaGetLastError());
  for (int l = 0; l + 1 < mg->num_levels; ++l) {
    const double* vf = (l == 0) ? values0 : mg->values[l];
    const int32_t* fi = mg->dims[l];
    const int32_t* co = mg->dims[l + 1];
    const cpfem_sell_t& C = mg->sell[l + 1];
    // x pass: fine SELL -> scratch[0] (co.x, fi.y, fi.z); y pass -> scratch[1] (co.x, co.y,
    // fi.z); z pass -> the coarse SELL
    const int64_t n1 = (int64_t)co[0] * fi[1] * fi[2], n2 = (int64_t)co[0] * co[1] * fi[2];
    const int64_t n3 = (int64_t)co[0] * co[1] * co[2];
    k_mg_rap_dir<<<(unsigned)ceil_div(27 * n1, 256), 256, 0, s>>>(0, fi[0], fi[1], fi[2], co[0], fi[1], fi[2],
                                                                   mg->sell[l], vf, mg->slot[l], nullptr,
                                                                   (l == 0) ? mg->free_dof : nullptr,
                                                                   mg->scratch[0], C, nullptr, nullptr);
    CPFEM_CUDA_TRY(cudaGetLastError());
    k_mg_rap_dir<<<(unsigned)ceil_div(27 * n2, 256), 256, 0, s>>>(1, co[0], fi[1], fi[2], co[0], co[1], fi[2],
                                                                   mg->sell[l], nullptr, nullptr, mg->scratch[0],
                                                                   nullptr, mg->scratch[1], C, nullptr, nullptr);
    CPFEM_CUDA_TRY(cudaGetLastError());
    k_mg_rap_dir<<<(unsigned)ceil_div(27 * n3, 256), 256, 0, s>>>(2, co[0], co[1], fi[2], co[0], co[1], co[2],
                                                                   mg->sell[l], nullptr, nullptr, mg->scratch[1],
                                                                   nullptr, nullptr, C, mg->slot[l + 1],
                                                                   mg->values[l + 1]);
    CPFEM_CUDA_TRY(cudaGetLastError());
    k_precond_setup<false><<<(unsigned)ceil_div(C.num_nodes, 128), 128, 0, s>>>(C, mg->values[l + 1], 2,
                                                                                mg->minv[l + 1]);
    CPFEM_CUDA_TRY(cudaGetLastError());
  }
  if (mg->precision == 1) {
    // the FP32 V-cycle's coarse operators: rounded copies of the FP64 ones (level 0 reads
    // the system's values directly)
    for (int l = 0; l < mg->num_levels; ++l) {
      const cpfem_sell_t& S = mg->sell[l];
      if (l > 0) {
        k_to_f32<<<1216, 256, 0, s>>>(mg->values[l], mg->values32[l], 0, S.group_off + S.num_groups);
        CPFEM_CUDA_TRY(cudaGetLastError());
      }
      const int64_t nm = 9 * (int64_t)S.num_nodes;
      k_to_f32<<<(unsigned)std::min<int64_t>(ceil_div(nm, 256), 1216), 256, 0, s>>>(mg->minv[l], mg->minv32[l], nm,
                                                                                   nullptr);
      CPFEM_CUDA_TRY(cudaGetLastError());
    }
  }
  return CPFEM_OK;
}

size_t cpfem_bicgstab_workspace_bytes(int32_t num_nodes) { return carve(nullptr, num_nodes, nullptr); }

int cpfem_bicgstab_last_stats(double* out) {
  CPFEM_REQUIRE(out != nullptr, "out is null");
  out[0] = (double)g_last_solve.k;
  out[1] = g_last_solve.rs;
  out[2] = g_last_solve.atol2;
  out[3] = g_last_solve.rho;
  out[4] = g_last_solve.alpha;
  out[5] = g_last_solve.omega;
  out[6] = (double)g_last_solve.restarts;
  return CPFEM_OK;
}

int cpfem_bicgstab_last_stats_ex(double* out, int32_t n) {
  CPFEM_REQUIRE(out != nullptr && n >= 0, "bad stats arguments");
  const double v[9] = {(double)g_last_solve.k, g_last_solve.rs, g_last_solve.atol2, g_last_solve.rho,
                       g_last_solve.alpha, g_last_solve.omega, (double)g_last_solve.restarts,
                       g_last_solve.true_rs, g_last_solve.bb};
  for (int32_t i = 0; i < n && i < 9; ++i) out[i] = v[i];
  return CPFEM_OK;
}

int cpfem_bicgstab_ex(const cpfem_sell_t* sell, const double* values, const double* b, double* x,
                      const cpfem_krylov_opts_t* opts, void* workspace, int32_t* info, void* stream) {
  CPFEM_REQUIRE(info != nullptr, "info is null");
  info[0] = 0;
  info[1] = 1;
  CPFEM_REQUIRE(opts != nullptr, "opts is null");
  CPFEM_REQUIRE(sell_ok(sell), "bad layout");
  if (sell->num_nodes == 0) return CPFEM_OK;
  CPFEM_REQUIRE(values && b && x && workspace, "bad bicgstab arguments");
  CPFEM_REQUIRE(((uintptr_t)workspace & 255) == 0, "workspace must be 256-byte aligned");
  CPFEM_REQUIRE(opts->precond >= 0 && opts->precond <= 3, "precond must be 0, 1, 2 or 3");
  if (opts->precond == 3) {
    CPFEM_REQUIRE(!opts->transpose || sell->tpos != nullptr, "a transposed multigrid solve needs tpos");
    const int rc = mg_check(opts->mg, sell);
    if (rc != CPFEM_OK) return rc;
  }
  CPFEM_REQUIRE(opts->maxiter >= 0, "maxiter must be >= 0");
  CPFEM_REQUIRE(opts->max_restarts >= 0, "max_restarts must be >= 0");
  CPFEM_REQUIRE(opts->grid_blocks >= 0, "grid_blocks must be >= 0");
  CPFEM_REQUIRE(!opts->transpose || sell->tpos != nullptr, "transpose needs tpos");
  CPFEM_REQUIRE(!(opts->flags & kKrylovDeferred) || opts->report != nullptr, "a deferred report needs opts.report");
  cudaStream_t s = (cudaStream_t)stream;
  if (opts->transpose)
    return run_bicgstab<true>(*sell, values, b, x, opts->precond, opts->tol, opts->atol, opts->maxiter, workspace,
                              info, s, opts->max_restarts, opts->mg, opts->grid_blocks, opts->flags, opts->report);
  return run_bicgstab<false>(*sell, values, b, x, opts->precond, opts->tol, opts->atol, opts->maxiter, workspace,
                             info, s, opts->max_restarts, opts->mg, opts->grid_blocks, opts->flags, opts->report);
}

int cpfem_bicgstab(const cpfem_sell_t* sell, const double* values, const double* b, double* x, int32_t precond,
                   int32_t transpose, double tol, double atol, int32_t maxiter, void* workspace, int32_t* info,
                   void* stream) {
  CPFEM_REQUIRE(precond >= 0 && precond <= 2, "precond must be 0, 1 or 2 (multigrid: cpfem_bicgstab_ex)");
  const cpfem_krylov_opts_t o = {precond, transpose, maxiter, 0, tol, atol, nullptr, 0, 0, nullptr};
  return cpfem_bicgstab_ex(sell, values, b, x, &o, workspace, info, stream);
}

}  // extern "C"

// ---- ragged batch: teams of blocks, one instance per team --------------------------------
// A ragged batch (instances of very different sizes and iteration counts) is split over the
// co-resident blocks of one cooperative launch.  When the batch has no more instances than
// blocks, every instance gets a team of consecutive blocks sized by its estimated work
// (nodes x expected iterations), so a 24^3 RVE and an 8^3 RVE finish at about the same
// time; a team crosses its dependencies with its own bounded barrier and reduces its dot
// products in a fixed block order.  With more instances than blocks, every block is a team
// of one that pulls instances from a queue, largest first.
namespace cpfem {

constexpr int kMinNodesPerBlock = 256;

struct RTeam {
  int first;   // first block of the team
  int nb;      // blocks in the team
  int job;     // the team's job, or -1: pull jobs from the queue (nb == 1)
  int pad;
};

struct RJob {
  int inst;
  int pad;
  int64_t n0, n1;
};

struct RWork {
  double *r, *rhat, *p, *q, *s, *t, *phat, *shat, *minv;
  double* partials;      // 2 buffers x 4 values x kMaxBlocks, by block id
  int* team_of_block;    // kMaxBlocks
  RTeam* teams;          // kMaxBlocks
  GridSync* tsync;       // one barrier per team
  RJob* jobs;            // at most num_nodes (every listed instance owns a node)
  int32_t* info;         // 2 per job
  unsigned int* queue;
  int* error;
};

static size_t carve_ragged(void* base, int64_t n_nodes, RWork* w) {
  const int64_t n = 3 * n_nodes;
  const int64_t nj = std::max<int64_t>(n_nodes, 1);
  char* p = (char*)base;
  size_t off = 0;
  auto take = [&](size_t bytes) {
    char* q = p ? p + off : nullptr;
    off += align256(bytes);
    return q;
  };
  RWork tmp;
  double** vecs[] = {&tmp.r, &tmp.rhat, &tmp.p, &tmp.q, &tmp.s, &tmp.t, &tmp.phat, &tmp.shat};
  for (double** v : vecs) *v = (double*)take(sizeof(double) * n);
  tmp.minv = (double*)take(sizeof(double) * 9 * n_nodes);
  tmp.partials = (double*)take(sizeof(double) * 2 * 4 * kMaxBlocks);
  tmp.team_of_block = (int*)take(sizeof(int) * kMaxBlocks);
  tmp.teams = (RTeam*)take(sizeof(RTeam) * kMaxBlocks);
  tmp.tsync = (GridSync*)take(sizeof(GridSync) * kMaxBlocks);
  tmp.jobs = (RJob*)take(sizeof(RJob) * nj);
  tmp.info = (int32_t*)take(sizeof(int32_t) * 2 * nj);
  tmp.queue = (unsigned int*)take(sizeof(unsigned int));
  tmp.error = (int*)take(sizeof(int));
  if (w) *w = tmp;
  return off;
}

__device__ __forceinline__ bool team_barrier(GridSync* gs, unsigned int nb, unsigned int& gen, int* gerr) {
  return counted_barrier(gs, nb, gen, gerr);
}

// Team-wide sums of NV values: block sum, then (teams of several blocks) publish, barrier
// and add the team's partials in block order.  Every block of the team gets the same bits.
template <int NV>
__device__ __forceinline__ bool team_reduce(double (&v)[NV], double* partials, int first, int nb, GridSync* gs,
                                            unsigned int& gen, int* gerr, double* smem, double* bcast) {
  block_sum<NV>(v, smem);
  bool ok = true;
  if (nb == 1) {
    if (threadIdx.x == 0)
#pragma unroll
      for (int k = 0; k < NV; ++k) bcast[k] = v[k];
  } else {
    if (threadIdx.x == 0)
#pragma unroll
      for (int k = 0; k < NV; ++k) partials[k * kMaxBlocks + blockIdx.x] = v[k];
    ok = team_barrier(gs, (unsigned)nb, gen, gerr);
    if (threadIdx.x < 32) {
      double acc[NV];
#pragma unroll
      for (int k = 0; k < NV; ++k) acc[k] = 0.0;
      for (int b = first + (int)threadIdx.x; b < first + nb; b += 32)
#pragma unroll
        for (int k = 0; k < NV; ++k) acc[k] += __ldcg(&partials[k * kMaxBlocks + b]);
      warp_sum<NV>(acc);
      if (threadIdx.x == 0)
#pragma unroll
        for (int k = 0; k < NV; ++k) bcast[k] = acc[k];
    }
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < NV; ++k) v[k] = bcast[k];
  __syncthreads();
  return ok;
}

__global__ void __launch_bounds__(kPThreads, 4) k_bicgstab_ragged(
    const cpfem_sell_t L, const double* __restrict__ vals, const double* __restrict__ b, double* __restrict__ x,
    RWork w, int precond, double tol, double atol, int maxiter, int n_jobs) {
  __shared__ double smem[4 * 32];
  __shared__ double bcast[4];
  __shared__ int s_job;
  const int team = w.team_of_block[blockIdx.x];
  const RTeam tm = w.teams[team];
  GridSync* gs = w.tsync + team;
  const int nb = tm.nb, first = tm.first;
  const int64_t tid = (int64_t)(blockIdx.x - first) * blockDim.x + threadIdx.x;
  const int64_t stride = (int64_t)nb * blockDim.x;
  unsigned int gen = 0u;
  int buf = 0;
  auto parts = [&]() {
    double* p = w.partials + (size_t)buf * 4 * kMaxBlocks;
    buf ^= 1;
    return p;
  };
  bool ok = true;
  for (int pass = 0; ok; ++pass) {
    int job;
    if (tm.job >= 0) {
      if (pass > 0) break;
      job = tm.job;
    } else {
      if (threadIdx.x == 0) s_job = (int)atomicAdd(w.queue, 1u);
      __syncthreads();
      job = s_job;
      __syncthreads();
    }
    if (job >= n_jobs) break;
    const RJob jb = w.jobs[job];
    const int64_t n0 = jb.n0, n1 = jb.n1;
    const int64_t a0 = ((n0 >> 5) << 5) + tid;   // group-aligned: a warp reads one sliced-ELL group

    double v2[2] = {0.0, 0.0};
    for (int64_t a = a0; a < n1; a += stride) {
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
    ok = team_reduce<2>(v2, parts(), first, nb, gs, gen, w.error, smem, bcast) && ok;
    const double atol2 = fmax(tol * tol * v2[0], atol * atol);
    double rs = v2[1], rho_new = v2[1], rho = 1.0, alpha = 1.0, omega = 1.0;
    int k = 0;
    while (ok && rs > atol2 && k < maxiter && k >= 0) {
      const double beta = rho_new / rho * alpha / omega;
      for (int64_t a = a0; a < n1; a += stride) {
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
      if (nb > 1) ok = team_barrier(gs, (unsigned)nb, gen, w.error) && ok;
      else __syncthreads();
      double v1[1] = {0.0};
      for (int64_t a = a0; a < n1; a += stride) {
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
      ok = team_reduce<1>(v1, parts(), first, nb, gs, gen, w.error, smem, bcast) && ok;
      alpha = rho_new / v1[0];
      double vs[1] = {0.0};
      for (int64_t a = a0; a < n1; a += stride) {
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
      ok = team_reduce<1>(vs, parts(), first, nb, gs, gen, w.error, smem, bcast) && ok;
      const bool early = vs[0] < atol2;
      double vt[2] = {0.0, 0.0};
      for (int64_t a = a0; a < n1; a += stride) {
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
      ok = team_reduce<2>(vt, parts(), first, nb, gs, gen, w.error, smem, bcast) && ok;
      omega = vt[0] / vt[1];
      double vr[2] = {0.0, 0.0};
      for (int64_t a = a0; a < n1; a += stride) {
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
      ok = team_reduce<2>(vr, parts(), first, nb, gs, gen, w.error, smem, bcast) && ok;
      int kn = (omega == 0.0 || alpha == 0.0) ? -11 : k + 1;
      if (rho_new == 0.0) kn = -10;
      k = kn;
      rho = rho_new;
      rho_new = vr[1];
      rs = vr[0];
    }
    if ((int)blockIdx.x == first && threadIdx.x == 0) {
      w.info[2 * job] = k;
      w.info[2 * job + 1] = (rs <= atol2) ? 1 : 0;
    }
  }
}

}  // namespace cpfem

extern "C" {

size_t cpfem_bicgstab_batched_workspace_bytes(int32_t num_nodes) {
  return cpfem::carve_ragged(nullptr, num_nodes, nullptr);
}

int cpfem_bicgstab_batched(const cpfem_sell_t* sell, const double* values, const double* b, double* x,
                           int32_t precond, double tol, double atol, int32_t maxiter, int32_t num_instances,
                           const int32_t* node_off, int32_t num_active, const int32_t* active,
                           const double* weights, void* workspace, int32_t* info, void* stream) {
  using namespace cpfem;
  CPFEM_REQUIRE(sell_ok(sell), "bad layout");
  CPFEM_REQUIRE(num_instances >= 0 && num_active >= 0 && num_active <= num_instances, "bad instance counts");
  if (num_active == 0 || sell->num_nodes == 0) return CPFEM_OK;
  CPFEM_REQUIRE(values && b && x && active && node_off && workspace && info, "bad batched bicgstab arguments");
  CPFEM_REQUIRE(((uintptr_t)workspace & 255) == 0, "workspace must be 256-byte aligned");
  CPFEM_REQUIRE(precond >= 0 && precond <= 2 && maxiter >= 0, "bad solver settings");
  CPFEM_REQUIRE(node_off[0] >= 0 && node_off[num_instances] <= sell->num_nodes, "node_off outside the system");
  for (int32_t i = 0; i < num_instances; ++i)
    CPFEM_REQUIRE(node_off[i + 1] >= node_off[i], "node_off must be non-decreasing");
  // jobs: listed instances that own nodes, heaviest first
  std::vector<char> seen((size_t)num_instances, 0);
  std::vector<RJob> jobs;
  std::vector<double> wts;
  jobs.reserve((size_t)num_active);
  for (int32_t j = 0; j < num_active; ++j) {
    const int32_t inst = active[j];
    CPFEM_REQUIRE(inst >= 0 && inst < num_instances, "active instance out of range");
    CPFEM_REQUIRE(!seen[(size_t)inst], "an instance is listed twice");
    seen[(size_t)inst] = 1;
    const int64_t n0 = node_off[inst], n1 = node_off[inst + 1];
    if (n1 == n0) {
      info[2 * inst] = 0;
      info[2 * inst + 1] = 1;
      continue;
    }
    const double wt = weights ? weights[j] : std::pow((double)(n1 - n0), 4.0 / 3.0);
    CPFEM_REQUIRE(wt > 0.0 && std::isfinite(wt), "weights must be positive");
    jobs.push_back(RJob{inst, 0, n0, n1});
    wts.push_back(wt);
  }
  if (jobs.empty()) return CPFEM_OK;
  {
    std::vector<size_t> order(jobs.size());
    for (size_t i = 0; i < order.size(); ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t c) { return wts[a] > wts[c]; });
    std::vector<RJob> j2(jobs.size());
    std::vector<double> w2(jobs.size());
    for (size_t i = 0; i < order.size(); ++i) { j2[i] = jobs[order[i]]; w2[i] = wts[order[i]]; }
    jobs.swap(j2);
    wts.swap(w2);
  }
  const int nj = (int)jobs.size();
  cudaStream_t s = (cudaStream_t)stream;
  RWork w;
  carve_ragged(workspace, sell->num_nodes, &w);
  int dev = 0, sms = 0, per_sm = 0;
  CPFEM_CUDA_TRY(cudaGetDevice(&dev));
  CPFEM_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  CPFEM_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, (const void*)k_bicgstab_ragged, kPThreads, 0));
  if (per_sm < 1) {
    set_error("ragged BiCGSTAB kernel cannot be resident");
    return CPFEM_ERR_CUDA;
  }
  const int bmax = (int)std::min<int64_t>((int64_t)per_sm * sms, kMaxBlocks);
  std::vector<RTeam> teams;
  std::vector<int> team_of_block;
  if (nj <= bmax) {
    // static plan: one team per job, 1 block plus a share of the spare blocks by weight
    double wsum = 0.0;
    for (double v : wts) wsum += v;
    const int spare = bmax - nj;
    int next = 0;
    for (int j = 0; j < nj; ++j) {
      const int64_t cap = std::max<int64_t>(1, ceil_div(jobs[(size_t)j].n1 - jobs[(size_t)j].n0, kMinNodesPerBlock));
      int64_t k = 1 + (int64_t)std::floor((double)spare * wts[(size_t)j] / wsum);
      k = std::min<int64_t>(k, cap);
      teams.push_back(RTeam{next, (int)k, j, 0});
      for (int64_t c = 0; c < k; ++c) team_of_block.push_back(j);
      next += (int)k;
    }
  } else {
    for (int blk = 0; blk < bmax; ++blk) {
      teams.push_back(RTeam{blk, 1, -1, 0});
      team_of_block.push_back(blk);
    }
  }
  const int blocks = (int)team_of_block.size();
  CPFEM_CUDA_TRY(cudaMemcpyAsync(w.teams, teams.data(), sizeof(RTeam) * teams.size(), cudaMemcpyHostToDevice, s));
  CPFEM_CUDA_TRY(cudaMemcpyAsync(w.team_of_block, team_of_block.data(), sizeof(int) * (size_t)blocks,
                                 cudaMemcpyHostToDevice, s));
  CPFEM_CUDA_TRY(cudaMemcpyAsync(w.jobs, jobs.data(), sizeof(RJob) * (size_t)nj, cudaMemcpyHostToDevice, s));
  CPFEM_CUDA_TRY(cudaMemsetAsync(w.tsync, 0, sizeof(GridSync) * teams.size(), s));
  CPFEM_CUDA_TRY(cudaMemsetAsync(w.queue, 0, sizeof(unsigned int), s));
  CPFEM_CUDA_TRY(cudaMemsetAsync(w.error, 0, sizeof(int), s));
  if (precond != 0) {
    k_precond_setup<false><<<(unsigned)ceil_div(sell->num_nodes, 128), 128, 0, s>>>(*sell, values, precond, w.minv);
    CPFEM_CUDA_TRY(cudaGetLastError());
  }
  cpfem_sell_t Lc = *sell;
  const double* bb = b;
  double* xx = x;
  int pc = precond, mi = maxiter, njobs = nj;
  double tl = tol, at = atol;
  void* args[] = {&Lc, &values, &bb, &xx, &w, &pc, &tl, &at, &mi, &njobs};
  CPFEM_CUDA_TRY(cudaLaunchCooperativeKernel((const void*)k_bicgstab_ragged, dim3((unsigned)blocks), dim3(kPThreads),
                                             args, 0, s));
  std::vector<int32_t> out((size_t)(2 * nj));
  int err = 0;
  CPFEM_CUDA_TRY(cudaMemcpyAsync(out.data(), w.info, sizeof(int32_t) * out.size(), cudaMemcpyDeviceToHost, s));
  CPFEM_CUDA_TRY(cudaMemcpyAsync(&err, w.error, sizeof(int), cudaMemcpyDeviceToHost, s));
  CPFEM_CUDA_TRY(cudaStreamSynchronize(s));
  for (int j = 0; j < nj; ++j) {
    info[2 * jobs[(size_t)j].inst] = out[(size_t)(2 * j)];
    info[2 * jobs[(size_t)j].inst + 1] = out[(size_t)(2 * j + 1)];
  }
  if (err) {
    set_error("ragged BiCGSTAB team barrier timed out");
    return CPFEM_ERR_SOLVE;
  }
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
static_assert(carve_bytes(kNoAllocMaxNodes) <= CPFEM_NOALLOC_SCRATCH_BYTES,
              "the allocation-free scratch is smaller than the solver's layout for CPFEM_NOALLOC_MAX_NODES");

static std::mutex g_noalloc_mutex;
static void* g_noalloc_ptr[256] = {nullptr};

// Device address of the scratch on the current device.  Host code must not use the
// symbol's name as an address: it is a host-side stand-in.  Resolved once per device index
// and kept: the address belongs to that device's primary context (the runtime API's).
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
  CPFEM_REQUIRE(noalloc_bytes_needed() == carve_bytes(kNoAllocMaxNodes) &&
                    noalloc_bytes_needed() <= sizeof(g_noalloc_scratch),
                "scratch smaller than its layout");
  void* ws = nullptr;
  int rc = noalloc_scratch(&ws);
  if (rc != CPFEM_OK) return rc;
  // run_bicgstab clears the barrier words and writes every vector before reading it
  return cpfem_bicgstab(sell, values, b, x, precond, transpose, tol, atol, maxiter, ws, info, stream);
}
