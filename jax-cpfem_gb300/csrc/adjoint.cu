// Per-Gauss-point backward pass of one load step (the discrete adjoint of the load-step
// sequence; reference: ad_wrapper / implicit_vjp, crystal_plasticity_OR_design/solver.py:801-874,
// and jax.grad through newton_solver's custom_jvp, models_copper.py:251-259).
#include "cpfem_common.cuh"
#include "gp_adjoint.cuh"

namespace cpfem {

constexpr int kVjpK = 4;   // tangent directions per dual sweep

template <int NS>
__global__ void __launch_bounds__(64) k_gp_vjp(const MatDev m, const cpfem_vjp_args_t a) {
  const int64_t gp = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t G = a.num_gp;
  if (gp >= G) return;
  const int64_t e = gp >> 3;
  const int32_t* cn = a.cells + e * 8;
  const double* sg = a.shape_grads + gp * 24;
  // every index gathered from the inputs is checked; a bad one is recorded, not read
  bool bad = false;
#pragma unroll
  for (int b = 0; b < 8; ++b) bad = bad || cn[b] < 0 || cn[b] >= a.num_nodes;
  const int64_t ri = a.rot_idx[gp];
  const int64_t pi = (a.param_idx != nullptr) ? a.param_idx[gp] : 0;
  bad = bad || ri < 0 || ri >= a.num_rot || pi < 0 || pi >= a.num_param;
  if (bad) {
    if (a.status != nullptr) atomicOr(a.status, CPFEM_GP_BOUNDS);
    return;
  }
  // kinematics at the checkpointed solution
  double F[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) F[k] = (k % 4 == 0) ? 1.0 : 0.0;
#pragma unroll
  for (int b = 0; b < 8; ++b) {
    const int64_t nb = cn[b];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int J = 0; J < 3; ++J) F[3 * i + J] = fma(a.u[3 * nb + i], sg[3 * b + J], F[3 * i + J]);
  }
  double Fpi[9], R[9], th[5], g[NS], ig[NS];
#pragma unroll
  for (int k = 0; k < 9; ++k) Fpi[k] = a.fpi[k * G + gp];
#pragma unroll
  for (int k = 0; k < 9; ++k) R[k] = a.rot_table[9 * ri + k];
#pragma unroll
  for (int k = 0; k < 5; ++k) th[k] = a.param_table[5 * pi + k];
  Cub cc{m.C11, m.C12, m.C44};
  if (a.elastic_table != nullptr) {
    cc.C11 = a.elastic_table[3 * pi];
    cc.C12 = a.elastic_table[3 * pi + 1];
    cc.C44 = a.elastic_table[3 * pi + 2];
  }
#pragma unroll
  for (int s = 0; s < NS; ++s) {
    g[s] = a.g[s * G + gp];
    ig[s] = 1.0 / g[s];
  }
  // recompute the converged local state from the checkpoint (u, Fp^-1, g and, if kept,
  // the converged S as the local Newton's start)
  double A[9], AR[9], Ct[9];
  mm3(F, Fpi, A);
  mm3(A, R, AR);
  mm3_at(AR, AR, Ct);
  const double cdt = m.ao * a.dt;
  GPSolve<NS> st;
  if (a.s_start != nullptr) {
    double s0[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) s0[k] = a.s_start[k * G + gp];
    cp_local_newton<NS>(m, cc, Ct, ig, cdt, 1.0 / th[3], st, s0);
  } else {
    cp_local_newton<NS>(m, cc, Ct, ig, cdt, 1.0 / th[3], st);
  }
  // output cotangents
  constexpr int NY = YOut<NS>::kN;
  double ybar[NY];
#pragma unroll
  for (int o = 0; o < NY; ++o) ybar[o] = 0.0;
  if (a.cell_sig_bar != nullptr) {
    double wsum = 0.0;
#pragma unroll
    for (int q = 0; q < 8; ++q) wsum += a.jxw[e * 8 + q];
    const double wq = a.jxw[gp] / wsum;
#pragma unroll
    for (int c = 0; c < 9; ++c) ybar[YOut<NS>::kSig + c] = a.cell_sig_bar[e * 9 + c] * wq;
  }
  if (a.fpi_bar != nullptr)
#pragma unroll
    for (int c = 0; c < 9; ++c) ybar[YOut<NS>::kFp + c] = a.fpi_bar[c * G + gp];
  if (a.g_bar != nullptr)
#pragma unroll
    for (int s = 0; s < NS; ++s) ybar[YOut<NS>::kG + s] = a.g_bar[s * G + gp];
  if (a.mode == 2 && a.mu != nullptr) {
    // P cotangent of the equilibrium term: -JxW * grad(mu)
    const double w = a.jxw[gp];
#pragma unroll
    for (int b = 0; b < 8; ++b) {
      const int64_t nb = cn[b];
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int J = 0; J < 3; ++J)
          ybar[YOut<NS>::kP + 3 * i + J] = fma(-w * a.mu[3 * nb + i], sg[3 * b + J], ybar[YOut<NS>::kP + 3 * i + J]);
    }
  }
  constexpr int NX = XIn<NS>::kN;
  double xbar[NX];
  int dirs[NX];
  int ndir = 0;
  if (a.mode == 1) {
#pragma unroll
    for (int k = 0; k < 9; ++k) dirs[ndir++] = XIn<NS>::kF + k;
  } else {
    for (int k = XIn<NS>::kFp; k < NX; ++k) dirs[ndir++] = k;
  }
  const bool ok = cp_vjp<NS, kVjpK>(m, cc, cdt, st.s, F, Fpi, g, R, th, ybar, dirs, ndir, xbar);
  if (a.status != nullptr) {
    int bits = 0;
    if (!(st.rn <= m.local_tol)) bits |= CPFEM_GP_MAXITER;
    if (!ok || !isfinite(st.rn)) bits |= CPFEM_GP_NONFINITE;
    if (bits) atomicOr(a.status, bits);
  }
  if (a.mode == 1) {
    if (a.f_bar != nullptr)
#pragma unroll
      for (int k = 0; k < 9; ++k) a.f_bar[k * G + gp] = xbar[XIn<NS>::kF + k];
  } else {
    if (a.fpi_bar_old != nullptr)
#pragma unroll
      for (int k = 0; k < 9; ++k) a.fpi_bar_old[k * G + gp] = xbar[XIn<NS>::kFp + k];
    if (a.g_bar_old != nullptr)
#pragma unroll
      for (int s = 0; s < NS; ++s) a.g_bar_old[s * G + gp] = xbar[XIn<NS>::kG + s];
    if (a.theta_bar != nullptr)
#pragma unroll
      for (int k = 0; k < 5; ++k) a.theta_bar[k * G + gp] = xbar[XIn<NS>::kTh + k];
    if (a.rot_bar != nullptr)
#pragma unroll
      for (int k = 0; k < 3; ++k) a.rot_bar[k * G + gp] = xbar[XIn<NS>::kW + k];
  }
}

}  // namespace cpfem

using namespace cpfem;

extern "C" int cpfem_gp_vjp(const cpfem_material_t* mat, const cpfem_vjp_args_t* args, void* stream) {
  CPFEM_REQUIRE(args != nullptr, "args is null");
  MatDev md;
  int rc = make_matdev(mat, &md);
  if (rc != CPFEM_OK) return rc;
  const cpfem_vjp_args_t& a = *args;
  if (a.num_gp == 0) return CPFEM_OK;
  CPFEM_REQUIRE(a.num_gp == (int64_t)a.num_cells * 8, "num_gp must be 8*num_cells");
  CPFEM_REQUIRE(a.mode == 1 || a.mode == 2, "mode must be 1 or 2");
  CPFEM_REQUIRE(a.u && a.cells && a.shape_grads && a.jxw && a.fpi && a.g && a.rot_table && a.rot_idx &&
                    a.param_table, "input pointer is null");
  CPFEM_REQUIRE(md.qmode == 0 || md.num_slip % 3 == 0, "qmode 1 needs num_slip % 3 == 0");
  CPFEM_REQUIRE(a.num_nodes > 0 && a.num_rot > 0 && a.num_param > 0, "table sizes must be given");
  const int threads = 64;
  const unsigned blocks = (unsigned)ceil_div(a.num_gp, threads);
  cudaStream_t s = (cudaStream_t)stream;
  const void* fn = (md.num_slip == 12) ? (const void*)k_gp_vjp<12> : (const void*)k_gp_vjp<24>;
  // the dual-number sweeps need a large per-thread stack: make sure the limit covers it
  cudaFuncAttributes attr;
  CPFEM_CUDA_TRY(cudaFuncGetAttributes(&attr, fn));
  size_t limit = 0;
  CPFEM_CUDA_TRY(cudaDeviceGetLimit(&limit, cudaLimitStackSize));
  const size_t need = attr.localSizeBytes + 1024;
  if (limit < need) CPFEM_CUDA_TRY(cudaDeviceSetLimit(cudaLimitStackSize, need));
  if (md.num_slip == 12)
    k_gp_vjp<12><<<blocks, threads, 0, s>>>(md, a);
  else
    k_gp_vjp<24><<<blocks, threads, 0, s>>>(md, a);
  CPFEM_CUDA_TRY(cudaGetLastError());
  return CPFEM_OK;
}
