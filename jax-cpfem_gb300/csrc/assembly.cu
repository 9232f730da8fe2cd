// Constitutive pass, element assembly, Dirichlet row elimination and small vector
// kernels of the cpfem_gb300 C ABI.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>

#include "cpfem_common.cuh"
#include "gp_update.cuh"
#include "reduce.cuh"

namespace cpfem {

static thread_local std::string g_last_error;

void set_error(const std::string& msg) { g_last_error = msg; }

int make_matdev(const cpfem_material_t* m, MatDev* o) {
  CPFEM_REQUIRE(m != nullptr && o != nullptr, "material is null");
  CPFEM_REQUIRE(m->num_slip == 12 || m->num_slip == 24, "num_slip must be 12 or 24");
  CPFEM_REQUIRE(m->qmode == 0 || m->qmode == 1, "qmode must be 0 or 1");
  CPFEM_REQUIRE(m->max_sub_step >= 1 && m->max_iter >= 1, "max_sub_step and max_iter must be >= 1");
  std::memset(o, 0, sizeof(*o));
  o->num_slip = m->num_slip;
  o->qmode = m->qmode;
  o->max_sub_step = m->max_sub_step;
  o->max_iter = m->max_iter;
  o->local_tol = m->local_tol;
  o->ao = m->ao;
  o->C11 = m->C11;
  o->C12 = m->C12;
  o->C44 = m->C44;
  for (int a = 0; a < m->num_slip; ++a) {
    const double* d = m->slip_d[a];
    const double* n = m->slip_n[a];
    for (int i = 0; i < 3; ++i) {
      o->d[a][i] = d[i];
      o->n[a][i] = n[i];
      for (int j = 0; j < 3; ++j) o->p9[a][3 * i + j] = d[i] * n[j];
    }
    o->pv[a][0] = d[0] * n[0];
    o->pv[a][1] = d[1] * n[1];
    o->pv[a][2] = d[2] * n[2];
    o->pv[a][3] = d[1] * n[2] + d[2] * n[1];
    o->pv[a][4] = d[0] * n[2] + d[2] * n[0];
    o->pv[a][5] = d[0] * n[1] + d[1] * n[0];
    for (int i = 0; i < 3; ++i) {
      o->d32[a][i] = (float)o->d[a][i];
      o->n32[a][i] = (float)o->n[a][i];
    }
    for (int k = 0; k < 6; ++k) o->pv32[a][k] = (float)o->pv[a][k];
  }
  return CPFEM_OK;
}

// ------------------------------------------------------------------------------------
// Constitutive pass: one thread per Gauss point.
// ------------------------------------------------------------------------------------
struct TanIn {
  double F[9], G[9], H[9], W[9], Y[9];
};

// The FP64 consistent tangent where the FP32 one's scale test fails: out of line, so the
// FP32-tangent kernel's hot code stays small.
template <int NS, class StoreCol>
__device__ __noinline__ void cp_tangent_f64_cold(const MatDev& m, Cub cc, TanIn in, GPSolve<NS> st, double idet,
                                                 StoreCol store) {
  cp_tangent<NS>(m, cc, in.F, in.G, st, in.H, in.W, in.Y, idet, store);
}

// TMODE: 0 no tangent, 1 FP64 tangent, 2 FP32 tangent (FP64 where the scale test fails)
// stored in FP64, 3 the same stored in FP32 (tangent32)
template <int NS, int TMODE>
__global__ void __launch_bounds__(128) k_gp_eval(const MatDev m, const cpfem_gp_args_t a) {
  const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t G = a.num_gp;
  int64_t gp = tid;
  if (a.cell_list != nullptr) {
    if (tid >= 8 * (int64_t)a.num_listed) return;
    const int64_t c = a.cell_list[tid >> 3];
    if (c < 0 || c >= a.num_cells) {
      atomicOr(a.status, CPFEM_GP_BOUNDS);
      return;
    }
    gp = 8 * c + (tid & 7);
  } else if (a.order != nullptr) {
    if (tid >= G) return;
    gp = a.order[tid];
    if (gp < 0 || gp >= G) {
      atomicOr(a.status, CPFEM_GP_BOUNDS);
      return;
    }
  }
  if (gp >= G) return;

  double F[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) F[k] = (k % 4 == 0) ? 1.0 : 0.0;
  if (a.u != nullptr) {
    // u_grad = sum_b u_b (x) dN_b/dX at this quad (models_copper.py:277-278)
    const int64_t e = gp >> 3;
    const int32_t* cn = a.cells + e * 8;
    const double* sg = a.shape_grads + gp * 24;
#pragma unroll
    for (int b = 0; b < 8; ++b) {
      const int64_t nb = cn[b];
      const double u0 = a.u[3 * nb], u1 = a.u[3 * nb + 1], u2 = a.u[3 * nb + 2];
      const double g0 = sg[3 * b], g1 = sg[3 * b + 1], g2 = sg[3 * b + 2];
      F[0] = fma(u0, g0, F[0]); F[1] = fma(u0, g1, F[1]); F[2] = fma(u0, g2, F[2]);
      F[3] = fma(u1, g0, F[3]); F[4] = fma(u1, g1, F[4]); F[5] = fma(u1, g2, F[5]);
      F[6] = fma(u2, g0, F[6]); F[7] = fma(u2, g1, F[7]); F[8] = fma(u2, g2, F[8]);
    }
  } else {
#pragma unroll
    for (int k = 0; k < 9; ++k) F[k] += a.u_grad[k * G + gp];
  }
  double Fpi[9], R[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) Fpi[k] = a.fpi[k * G + gp];
  const int64_t ri = a.rot_idx[gp];
#pragma unroll
  for (int k = 0; k < 9; ++k) R[k] = a.rot_table[9 * ri + k];
  const int64_t pi = (a.param_idx != nullptr) ? a.param_idx[gp] : 0;
  const double gss_a = a.param_table[5 * pi + 0];
  const double hh = a.param_table[5 * pi + 1];
  const double t_sat = a.param_table[5 * pi + 2];
  const double xm = a.param_table[5 * pi + 3];
  const double rq = a.param_table[5 * pi + 4];
  Cub cc{m.C11, m.C12, m.C44};
  if (a.elastic_table != nullptr) {
    cc.C11 = a.elastic_table[3 * pi];
    cc.C12 = a.elastic_table[3 * pi + 1];
    cc.C44 = a.elastic_table[3 * pi + 2];
  }

  double g[NS], ig[NS];
#pragma unroll
  for (int s = 0; s < NS; ++s) {
    g[s] = a.g[s * G + gp];
    ig[s] = 1.0 / g[s];
  }
  double A[9], AR[9], Ct[9];
  mm3(F, Fpi, A);
  mm3(A, R, AR);
  mm3_at(AR, AR, Ct);

  GPSolve<NS> st;
  const bool predict = a.s_warm != nullptr && a.s_dsdf != nullptr && a.s_f != nullptr;
  if (a.s_warm != nullptr) {
    double s0[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) s0[k] = a.s_warm[k * G + gp];
    if (predict && (a.local_flags & 1)) {
      // first-order prediction from where s_warm converged: s0 += ds/dF : (F - F_then)
#pragma unroll
      for (int kl = 0; kl < 9; ++kl) {
        const double dF = F[kl] - a.s_f[kl * G + gp];
#pragma unroll
        for (int k = 0; k < 6; ++k) s0[k] = fma(a.s_dsdf[(6 * kl + k) * G + gp], dF, s0[k]);
      }
    }
    cp_local_newton<NS>(m, cc, Ct, ig, m.ao * a.dt, 1.0 / xm, st, s0, (a.local_flags & 2) != 0);
    if (st.rn <= m.local_tol) {
#pragma unroll
      for (int k = 0; k < 6; ++k) a.s_warm[k * G + gp] = st.s[k];
      if (predict)
#pragma unroll
        for (int kl = 0; kl < 9; ++kl) a.s_f[kl * G + gp] = F[kl];
    }
  } else {
    cp_local_newton<NS>(m, cc, Ct, ig, m.ao * a.dt, 1.0 / xm, st, nullptr, (a.local_flags & 2) != 0);
  }
  if (a.status != nullptr) {
    int bits = 0;
    if (!(st.rn <= m.local_tol)) bits |= CPFEM_GP_MAXITER;
    if (!isfinite(st.rn)) bits |= CPFEM_GP_NONFINITE;
    if (bits) atomicOr(a.status, bits);
  }

  double Gm[9], H[9], W[9], Y[9], P[9], idet;
  mm3(Fpi, R, Gm);
  cp_stress<NS>(F, Gm, st, H, W, Y, idet, P);
  const double w = (a.weight_jxw && a.jxw != nullptr) ? a.jxw[gp] : 1.0;

  // every output but the tangent first, so that the tangent computation (the register-
  // heaviest part) runs with only what it needs live
  if (a.pk1 != nullptr)
#pragma unroll
    for (int c = 0; c < 9; ++c) a.pk1[c * G + gp] = P[c] * w;
  if (a.stress != nullptr) {
    // sigma = P F^T / det F (models_copper.py:307-308)
    double sig[9];
    mm3_bt(P, F, sig);
    const double idf = w / det3(F);
#pragma unroll
    for (int c = 0; c < 9; ++c) a.stress[c * G + gp] = sig[c] * idf;
  }
  if (a.fpi_new != nullptr) {
    double Fn[9];
    mm3_bt(H, R, Fn);  // Fp^-1_old (I - R L R^T) = H R^T
#pragma unroll
    for (int c = 0; c < 9; ++c) a.fpi_new[c * G + gp] = Fn[c];
  }
  if (a.slip_new != nullptr)
#pragma unroll
    for (int s = 0; s < NS; ++s) a.slip_new[s * G + gp] = a.slip[s * G + gp] + st.dg[s];
  if (a.g_new != nullptr) {
    double gn[NS];
    cp_hardening<NS>(m, g, st.dg, hh, t_sat, gss_a, rq, gn);
#pragma unroll
    for (int s = 0; s < NS; ++s) a.g_new[s * G + gp] = gn[s];
  }
  if (a.s_out != nullptr) {
    double Sl[9], T1[9], Sg[9];
    Sl[0] = st.s[0]; Sl[4] = st.s[1]; Sl[8] = st.s[2];
    Sl[5] = Sl[7] = st.s[3];
    Sl[2] = Sl[6] = st.s[4];
    Sl[1] = Sl[3] = st.s[5];
    mm3(R, Sl, T1);
    mm3_bt(T1, R, Sg);
#pragma unroll
    for (int c = 0; c < 9; ++c) a.s_out[c * G + gp] = Sg[c];
  }
  if (a.iters != nullptr) a.iters[gp] = st.iters;
  if (TMODE != 0 && (a.tangent != nullptr || a.tangent32 != nullptr)) {
    const bool keep_dsdf = predict && st.rn <= m.local_tol;
    // columns arrive in the precision they were formed in; FP32 storage (tangent32)
    // takes an FP32 column as it is.  Everything captured by value: the store may be handed
    // to an out-of-line function.
    float* const tan32 = a.tangent32;
    double* const tan64 = a.tangent;
    double* const dsdf_out = a.s_dsdf;
    auto store = [=](int kl, const auto* col, const auto* dsdf) {
      if constexpr (TMODE == 3) {
        const float w32 = f32_of(w);
#pragma unroll
        for (int c = 0; c < 9; ++c) tan32[(int64_t)(9 * c + kl) * G + gp] = to_f32(col[c]) * w32;
      } else {
#pragma unroll
        for (int c = 0; c < 9; ++c) tan64[(int64_t)(9 * c + kl) * G + gp] = to_f64(col[c]) * w;
      }
      if (keep_dsdf)
#pragma unroll
        for (int k = 0; k < 6; ++k) dsdf_out[(6 * kl + k) * G + gp] = to_f64(dsdf[k]);
    };
    if constexpr (TMODE >= 2) {
      if (tangent_f32_ok<NS>(st, cc)) {
        cp_tangent_t<NS, float>(m, cc, F, Gm, st, H, W, Y, idet, store);
      } else {
        // the FP64 tangent is the cold path here: out of line, inputs by value
        TanIn in;
#pragma unroll
        for (int k = 0; k < 9; ++k) {
          in.F[k] = F[k]; in.G[k] = Gm[k]; in.H[k] = H[k]; in.W[k] = W[k]; in.Y[k] = Y[k];
        }
        cp_tangent_f64_cold<NS>(m, cc, in, st, idet, store);
      }
    } else {
      cp_tangent<NS>(m, cc, F, Gm, st, H, W, Y, idet, store);
    }
  }
}

// ------------------------------------------------------------------------------------
// Element residual / tangent: one thread per (cell, node a) owns rows (a, 0..2).
// KT is the precision of the element stiffness arithmetic (FP64, or FP32 for a tangent
// that only serves as the Newton Jacobian), TT that of the stored tangent (FP32 storage
// goes with FP32 arithmetic); the residual is always FP64.
// ------------------------------------------------------------------------------------
template <typename KT>
__device__ __forceinline__ KT as_kt(double v) { return to_prec<KT>(v); }
template <typename KT>
__device__ __forceinline__ KT as_kt(float v);
template <>
__device__ __forceinline__ float as_kt<float>(float v) { return v; }

// SPLIT threads share a (cell, node a): thread h of them forms the blocks of neighbours
// b = h*8/SPLIT .. (h+1)*8/SPLIT - 1 (each recomputes the node's 27 tangent contractions),
// so a colour's launch has SPLIT times the threads; every block of the matrix is still
// written by one thread, in the same order.
template <bool WITH_K, bool ATOMIC, typename KT = double, typename TT = double, int SPLIT = 1>
__global__ void __launch_bounds__(128, SPLIT == 2 ? (sizeof(KT) == 4 ? 4 : 2) : 1) k_elem_assemble(int32_t E, const int32_t* __restrict__ clist,
                                                       int32_t ncl, const int32_t* __restrict__ cells,
                                                       const double* __restrict__ sg,
                                                       const int64_t* __restrict__ goff,
                                                       const uint8_t* __restrict__ epos,
                                                       const double* __restrict__ Pw,
                                                       const TT* __restrict__ Dw,
                                                       double* __restrict__ res,
                                                       double* __restrict__ vals) {
  static_assert(SPLIT == 1 || SPLIT == 2, "SPLIT must be 1 or 2");
  constexpr int NB = 8 / SPLIT;   // neighbours b per thread
  const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int h = (SPLIT == 2) ? (int)(tid & 1) : 0;
  const int64_t tn = (SPLIT == 2) ? (tid >> 1) : tid;
  const int64_t li = tn >> 3;
  const int a = (int)(tn & 7);
  if (li >= ncl) return;
  const int64_t e = (clist != nullptr) ? clist[li] : li;
  const int64_t G = (int64_t)E * 8;
  const int b0 = h * NB;
  KT K[3][3 * NB];
  double Rr[3] = {0.0, 0.0, 0.0};
  if (WITH_K) {
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int c = 0; c < 3 * NB; ++c) K[i][c] = KT(0);
  }
#pragma unroll 1
  for (int q = 0; q < 8; ++q) {
    const int64_t gp = e * 8 + q;
    const double* sgq = sg + gp * 24;
    const double ga0 = sgq[3 * a], ga1 = sgq[3 * a + 1], ga2 = sgq[3 * a + 2];
    if (h == 0)
#pragma unroll
      for (int i = 0; i < 3; ++i)
        Rr[i] = fma(Pw[(3 * i) * G + gp], ga0, fma(Pw[(3 * i + 1) * G + gp], ga1, fma(Pw[(3 * i + 2) * G + gp], ga2, Rr[i])));
    if (WITH_K) {
      const KT a0 = as_kt<KT>(ga0), a1 = as_kt<KT>(ga1), a2 = as_kt<KT>(ga2);
      KT Gm[27];
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int kL = 0; kL < 9; ++kL)
          Gm[9 * i + kL] = cp_fma(a0, as_kt<KT>(Dw[(int64_t)(9 * (3 * i + 0) + kL) * G + gp]),
                           cp_fma(a1, as_kt<KT>(Dw[(int64_t)(9 * (3 * i + 1) + kL) * G + gp]),
                                  a2 * as_kt<KT>(Dw[(int64_t)(9 * (3 * i + 2) + kL) * G + gp])));
#pragma unroll
      for (int bl = 0; bl < NB; ++bl) {
        const int b = b0 + bl;
        const KT gb0 = as_kt<KT>(sgq[3 * b]), gb1 = as_kt<KT>(sgq[3 * b + 1]), gb2 = as_kt<KT>(sgq[3 * b + 2]);
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
          for (int k = 0; k < 3; ++k)
            K[i][3 * bl + k] = cp_fma(Gm[9 * i + 3 * k], gb0, cp_fma(Gm[9 * i + 3 * k + 1], gb1,
                               cp_fma(Gm[9 * i + 3 * k + 2], gb2, K[i][3 * bl + k])));
      }
    }
  }
  const int64_t na = cells[e * 8 + a];
  // a conflict-free cell list (one colour) adds without atomics, in a fixed order
  if (res != nullptr && h == 0)
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      if (ATOMIC) atomicAdd(&res[3 * na + i], Rr[i]);
      else res[3 * na + i] += Rr[i];
    }
  if (WITH_K) {
    // sliced-ELL slot of (node na, neighbour b): 9*goff[g] + 32*(9*pos + 3i + k) + lane
    const int64_t base = 9 * goff[na >> 5] + (na & 31);
#pragma unroll
    for (int bl = 0; bl < NB; ++bl) {
      const int64_t pos = epos[e * 64 + 8 * a + b0 + bl];
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          double* v = &vals[base + 32 * (9 * pos + 3 * i + k)];
          if (ATOMIC) atomicAdd(v, to_f64(K[i][3 * bl + k]));
          else *v += to_f64(K[i][3 * bl + k]);
        }
    }
  }
}

// Row elimination for a list of unique Dirichlet dofs.
__global__ void k_dirichlet(int32_t nbc, const int32_t* __restrict__ dofs, const double* __restrict__ bvals,
                            const double* __restrict__ u, double* __restrict__ res, const cpfem_sell_t L,
                            double* __restrict__ vals) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nbc) return;
  const int64_t d = dofs[t];
  if (res != nullptr) {
    double r = (u != nullptr) ? u[d] : 0.0;
    res[d] = r - bvals[t];
  }
  if (vals != nullptr) {
    const int64_t na = d / 3;
    const int i = (int)(d % 3);
    const int64_t g = na >> 5;
    const int64_t base = 9 * L.group_off[g] + (na & 31);
    const int w = L.group_width[g];
    for (int j = 0; j < w; ++j)
#pragma unroll
      for (int k = 0; k < 3; ++k) vals[base + 32 * (9 * j + 3 * i + k)] = 0.0;
    vals[base + 32 * (9 * L.diag_slot[na] + 3 * i + i)] = 1.0;
  }
}

__global__ void k_bc_guess(int32_t nbc, const int32_t* __restrict__ dofs, const double* __restrict__ bvals,
                           const double* __restrict__ u, double* __restrict__ x0) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nbc) return;
  const int64_t d = dofs[t];
  x0[d] = bvals[t] - ((u != nullptr) ? u[d] : 0.0);
}

__global__ void k_cell_average(int32_t E, const double* __restrict__ jxw, const double* __restrict__ fw,
                               double* __restrict__ out) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= E) return;
  const int64_t G = (int64_t)E * 8;
  double wsum = 0.0;
#pragma unroll
  for (int q = 0; q < 8; ++q) wsum += jxw[e * 8 + q];
#pragma unroll
  for (int c = 0; c < 9; ++c) {
    double acc = 0.0;
#pragma unroll
    for (int q = 0; q < 8; ++q) acc += fw[c * G + e * 8 + q];
    out[e * 9 + c] = acc / wsum;
  }
}

__global__ void k_axpy(int64_t n, double alpha, const double* __restrict__ x, double* __restrict__ y) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] = fma(alpha, x[i], y[i]);
}

__global__ void __launch_bounds__(kVecThreads) k_dot(int64_t n, const double* __restrict__ x,
                                                      const double* __restrict__ y, double* result,
                                                      double* partials, unsigned int* counter) {
  __shared__ double smem[32];
  double v[1] = {0.0};
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    v[0] = fma(x[i], y[i], v[0]);
  if (grid_sum<1>(v, partials, counter, smem) && threadIdx.x == 0) *result = v[0];
}

// out[i] = x.y over entries [off[i], off[i+1]) -- one block per segment, fixed order.
__global__ void __launch_bounds__(256) k_segmented_dot(int32_t nseg, const int64_t* __restrict__ off,
                                                       const double* __restrict__ x, const double* __restrict__ y,
                                                       double* __restrict__ out) {
  __shared__ double smem[32];
  for (int seg = blockIdx.x; seg < nseg; seg += gridDim.x) {
    double v[1] = {0.0};
    for (int64_t i = off[seg] + threadIdx.x; i < off[seg + 1]; i += blockDim.x) v[0] = fma(x[i], y[i], v[0]);
    block_sum<1>(v, smem);
    if (threadIdx.x == 0) out[seg] = v[0];
    __syncthreads();
  }
}

template <int NS>
static int launch_gp(const MatDev& md, const cpfem_gp_args_t& a, cudaStream_t s) {
  const int threads = 128;
  const int64_t work = a.cell_list != nullptr ? 8 * (int64_t)a.num_listed : a.num_gp;
  if (work == 0) return CPFEM_OK;
  const unsigned blocks = (unsigned)ceil_div(work, threads);
  if (a.tangent32 != nullptr)
    k_gp_eval<NS, 3><<<blocks, threads, 0, s>>>(md, a);
  else if (a.tangent != nullptr && (a.local_flags & 4))
    k_gp_eval<NS, 2><<<blocks, threads, 0, s>>>(md, a);
  else if (a.tangent != nullptr)
    k_gp_eval<NS, 1><<<blocks, threads, 0, s>>>(md, a);
  else
    k_gp_eval<NS, 0><<<blocks, threads, 0, s>>>(md, a);
  CPFEM_CUDA_TRY(cudaGetLastError());
  return CPFEM_OK;
}

}  // namespace cpfem

using namespace cpfem;

extern "C" {

int cpfem_abi_version(void) { return CPFEM_ABI_VERSION; }

const char* cpfem_last_error(void) { return g_last_error.c_str(); }

int cpfem_gp_eval(const cpfem_material_t* mat, const cpfem_gp_args_t* args, void* stream) {
  CPFEM_REQUIRE(args != nullptr, "args is null");
  MatDev md;
  int rc = make_matdev(mat, &md);
  if (rc != CPFEM_OK) return rc;
  const cpfem_gp_args_t& a = *args;
  if (a.num_gp == 0) return CPFEM_OK;
  CPFEM_REQUIRE(a.num_gp > 0, "num_gp must be >= 0");
  CPFEM_REQUIRE(a.fpi && a.g && a.rot_table && a.rot_idx && a.param_table, "state/table pointer is null");
  CPFEM_REQUIRE(a.u != nullptr || a.u_grad != nullptr, "need u or u_grad");
  if (a.u != nullptr) {
    CPFEM_REQUIRE(a.cells && a.shape_grads, "u given without cells/shape_grads");
    CPFEM_REQUIRE(a.num_gp == (int64_t)a.num_cells * 8, "num_gp must be 8*num_cells with nodal u");
  }
  CPFEM_REQUIRE(!(a.weight_jxw && a.jxw == nullptr), "weight_jxw without jxw");
  CPFEM_REQUIRE(a.cell_list == nullptr || (a.u != nullptr && a.status != nullptr && a.num_listed >= 0 &&
                                           a.num_listed <= a.num_cells),
                "a cell list needs nodal u, a status word and 0 <= num_listed <= num_cells");
  CPFEM_REQUIRE(a.order == nullptr || (a.cell_list == nullptr && a.status != nullptr),
                "an evaluation order excludes a cell list and needs a status word");
  CPFEM_REQUIRE(a.slip_new == nullptr || a.slip != nullptr, "slip_new needs slip");
  CPFEM_REQUIRE(a.tangent32 == nullptr || (a.tangent == nullptr && (a.local_flags & 4)),
                "tangent32 needs local_flags bit 4 and excludes tangent");
  CPFEM_REQUIRE(md.qmode == 0 || md.num_slip % 3 == 0, "qmode 1 needs num_slip % 3 == 0");
  cudaStream_t s = (cudaStream_t)stream;
  if (md.num_slip == 12) return launch_gp<12>(md, a, s);
  return launch_gp<24>(md, a, s);
}

int cpfem_elem_assemble(int32_t num_cells, const int32_t* cells, const double* shape_grads,
                        const cpfem_sell_t* sell, const uint8_t* elem_pos, const int32_t* cell_list,
                        int32_t num_listed, const double* pk1_w, const double* tangent_w, double* residual,
                        double* values, void* stream) {
  return cpfem_elem_assemble_ex(num_cells, cells, shape_grads, sell, elem_pos, cell_list, num_listed, pk1_w,
                                tangent_w, residual, values, 0, stream);
}

int cpfem_elem_assemble_ex(int32_t num_cells, const int32_t* cells, const double* shape_grads,
                           const cpfem_sell_t* sell, const uint8_t* elem_pos, const int32_t* cell_list,
                           int32_t num_listed, const double* pk1_w, const void* tangent_w, double* residual,
                           double* values, int32_t k_precision, void* stream) {
  if (num_cells == 0) return CPFEM_OK;
  CPFEM_REQUIRE(num_cells > 0 && cells && shape_grads && pk1_w, "bad element arguments");
  CPFEM_REQUIRE((values == nullptr) == (tangent_w == nullptr), "values and tangent_w go together");
  CPFEM_REQUIRE(values == nullptr || (sell && sell->group_off && elem_pos), "values need the layout");
  CPFEM_REQUIRE(cell_list == nullptr || (num_listed >= 0 && num_listed <= num_cells), "bad cell list");
  CPFEM_REQUIRE(k_precision >= 0 && k_precision <= 2,
                "k_precision must be 0 (FP64), 1 (FP32 stiffness) or 2 (FP32 tangent and stiffness)");
  const int32_t ncl = (cell_list != nullptr) ? num_listed : num_cells;
  if (ncl == 0) return CPFEM_OK;
  const int threads = 128;
  cudaStream_t s = (cudaStream_t)stream;
  const int64_t* goff = (values != nullptr) ? sell->group_off : nullptr;
  const double* t64 = static_cast<const double*>(tangent_w);
  const float* t32 = static_cast<const float*>(tangent_w);
  // a colour's cell list adds without atomics (bitwise reproducible); no list: atomics.
  // The stiffness variants give each (cell, node) two threads (one colour of a structured
  // box is too few threads otherwise), the residual-only one a thread.
  auto run = [&](auto kernel, auto tangent, int split) {
    const unsigned blocks = (unsigned)ceil_div((int64_t)ncl * 8 * split, threads);
    kernel<<<blocks, threads, 0, s>>>(num_cells, cell_list, ncl, cells, shape_grads, goff, elem_pos, pk1_w,
                                      tangent, residual, values);
  };
  const bool listed = cell_list != nullptr;
  if (values == nullptr) {
    if (listed) run(k_elem_assemble<false, false>, (const double*)nullptr, 1);
    else run(k_elem_assemble<false, true>, (const double*)nullptr, 1);
  } else if (k_precision == 0) {
    if (listed) run(k_elem_assemble<true, false, double, double, 2>, t64, 2);
    else run(k_elem_assemble<true, true, double, double, 2>, t64, 2);
  } else if (k_precision == 1) {
    if (listed) run(k_elem_assemble<true, false, float, double, 2>, t64, 2);
    else run(k_elem_assemble<true, true, float, double, 2>, t64, 2);
  } else {
    if (listed) run(k_elem_assemble<true, false, float, float, 2>, t32, 2);
    else run(k_elem_assemble<true, true, float, float, 2>, t32, 2);
  }
  CPFEM_CUDA_TRY(cudaGetLastError());
  return CPFEM_OK;
}

int cpfem_apply_dirichlet(int32_t num_bc, const int32_t* bc_dofs, const double* bc_vals, const double* u,
                          double* residual, const cpfem_sell_t* sell, double* values, void* stream) {
  if (num_bc == 0) return CPFEM_OK;
  CPFEM_REQUIRE(num_bc > 0 && bc_dofs && bc_vals, "bad Dirichlet arguments");
  CPFEM_REQUIRE(values == nullptr || (sell && sell->group_off && sell->group_width && sell->diag_slot),
                "values need the layout");
  cpfem_sell_t L{};
  if (sell) L = *sell;
  k_dirichlet<<<(unsigned)ceil_div(num_bc, 128), 128, 0, (cudaStream_t)stream>>>(num_bc, bc_dofs, bc_vals, u,
                                                                                 residual, L, values);
  CPFEM_CUDA_TRY(cudaGetLastError());
  return CPFEM_OK;
}

int cpfem_bc_initial_guess(int64_t ndof, int32_t num_bc, const int32_t* bc_dofs, const double* bc_vals,
                           const double* u, double* x0, void* stream) {
  CPFEM_REQUIRE(ndof >= 0 && x0 != nullptr, "bad x0");
  cudaStream_t s = (cudaStream_t)stream;
  CPFEM_CUDA_TRY(cudaMemsetAsync(x0, 0, sizeof(double) * (size_t)ndof, s));
  if (num_bc > 0) {
    CPFEM_REQUIRE(bc_dofs && bc_vals, "bad Dirichlet arguments");
    k_bc_guess<<<(unsigned)ceil_div(num_bc, 128), 128, 0, s>>>(num_bc, bc_dofs, bc_vals, u, x0);
    CPFEM_CUDA_TRY(cudaGetLastError());
  }
  return CPFEM_OK;
}

int cpfem_cell_average(int32_t num_cells, const double* jxw, const double* field_w, double* out,
                       void* stream) {
  if (num_cells == 0) return CPFEM_OK;
  CPFEM_REQUIRE(num_cells > 0 && jxw && field_w && out, "bad cell-average arguments");
  k_cell_average<<<(unsigned)ceil_div(num_cells, 128), 128, 0, (cudaStream_t)stream>>>(num_cells, jxw,
                                                                                      field_w, out);
  CPFEM_CUDA_TRY(cudaGetLastError());
  return CPFEM_OK;
}

int cpfem_axpy(int64_t n, double alpha, const double* x, double* y, void* stream) {
  if (n == 0) return CPFEM_OK;
  CPFEM_REQUIRE(n > 0 && x && y, "bad axpy arguments");
  const unsigned blocks = (unsigned)std::min<int64_t>(ceil_div(n, 256), 4 * 152);
  k_axpy<<<blocks, 256, 0, (cudaStream_t)stream>>>(n, alpha, x, y);
  CPFEM_CUDA_TRY(cudaGetLastError());
  return CPFEM_OK;
}

int cpfem_segmented_dot(int32_t num_segments, const int64_t* offsets, const double* x, const double* y,
                        double* out, void* stream) {
  if (num_segments == 0) return CPFEM_OK;
  CPFEM_REQUIRE(num_segments > 0 && offsets && x && y && out, "bad segmented dot arguments");
  const unsigned blocks = (unsigned)std::min<int64_t>(num_segments, 8 * 152);
  k_segmented_dot<<<blocks, 256, 0, (cudaStream_t)stream>>>(num_segments, offsets, x, y, out);
  CPFEM_CUDA_TRY(cudaGetLastError());
  return CPFEM_OK;
}

size_t cpfem_dot_workspace_bytes(int64_t) { return 256 + sizeof(double) * kVecBlocks; }

int cpfem_dot(int64_t n, const double* x, const double* y, double* result, void* workspace, void* stream) {
  CPFEM_REQUIRE(n >= 0 && x && y && result && workspace, "bad dot arguments");
  CPFEM_REQUIRE(((uintptr_t)workspace & 255) == 0, "workspace must be 256-byte aligned");
  unsigned int* counter = (unsigned int*)workspace;
  double* partials = (double*)((char*)workspace + 256);
  cudaStream_t s = (cudaStream_t)stream;
  CPFEM_CUDA_TRY(cudaMemsetAsync(counter, 0, sizeof(unsigned int), s));
  k_dot<<<kVecBlocks, kVecThreads, 0, s>>>(n, x, y, result, partials, counter);
  CPFEM_CUDA_TRY(cudaGetLastError());
  return CPFEM_OK;
}

}  // extern "C"
