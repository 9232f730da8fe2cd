// Per-Gauss-point Kalidindi update, one thread per GP, everything in FP64 registers.
//
// The reference (singlecrystal_copper/models_copper.py:155-259) solves for the second
// Piola-Kirchhoff stress S with 9 unknowns in the global frame:
//   r(S) = S - C'(R) : (Fe^T Fe - I)/2,   Fe = F Fp^-1_old (I - sum_a dg_a R P_a R^T),
//   dg_a = ao dt |tau_a/g_a|^(1/m) sign(tau_a),  tau_a = S : R P_a R^T.
// Here the same Newton iterates are computed in the lattice frame with the 6 symmetric
// unknowns s = R^T S R (11,22,33,23,13,12).  For an orthonormal R the residual norm, the
// Newton step, the line search and the converged S are the reference's (the map is an
// orthogonal change of variables, and from S0 = 0 the 9-unknown iterates stay
// symmetric because C' : E is symmetric).  This costs a 6x6 rather than a 9x9 solve and
// needs neither the rotated C' nor the rotated Schmid tensors.
#pragma once

#include "cpfem_common.cuh"

namespace cpfem {

// x^e for x >= 0 and a non-negative integer e, by binary exponentiation.  The
// Kalidindi exponents 1/m - 1 and a are integers for every shipped material (1/m = 10,
// 20, 120; a = 2, 8), and this costs about 2 log2(e) FP64 multiplies against the ~100
// FP64 operations of a general pow.
CPFEM_HD double ipow(double x, int e) {
  double r = 1.0;
  while (e > 0) {
    if (e & 1) r *= x;
    x *= x;
    e >>= 1;
  }
  return r;
}

// The integer exponent to use for x^p, or -1 when p is not a small non-negative integer.
CPFEM_HD int int_exponent(double p) {
  return (p >= 0.0 && p <= 1024.0 && p == floor(p)) ? (int)p : -1;
}

CPFEM_HD double powe(double x, double p, int ie) { return (ie >= 0) ? ipow(x, ie) : pow(x, p); }

template <int NS>
struct GPSolve {
  double s[6];      // converged lattice-frame S (tensor components)
  double dg[NS];    // slip increments at s
  double kk[NS];    // d(dg)/d(tau) at s
  double B[9];      // I - L_p,lattice at s
  double M[9];      // Ct * B at s
  double rn;        // ||r|| at s
  int iters;
};

// Residual at s.  Ct = (F Fp^-1_old R)^T (F Fp^-1_old R) (symmetric, full 3x3).
template <int NS>
CPFEM_HD void cp_residual(const MatDev& m, const Cub& cc, const double* Ct, const double* ig,
                                            double cdt, double pexp, int ie1, const double* s, double* r,
                                            double& rn, double* dg, double* kk, double* B,
                                            double* M) {
  double L[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) L[k] = 0.0;
#pragma unroll
  for (int a = 0; a < NS; ++a) {
    const double tau = fma(s[0], m.pv[a][0], fma(s[1], m.pv[a][1], fma(s[2], m.pv[a][2],
                       fma(s[3], m.pv[a][3], fma(s[4], m.pv[a][4], s[5] * m.pv[a][5])))));
    const double x = tau * ig[a];
    const double ax = fabs(x);
    // |x|^(p-1): dg = cdt |x|^(p-1) x = cdt |x|^p sign(tau) (g > 0), and the derivative
    // p cdt |x|^(p-1) / g uses the same power.
    const double pw1 = (ax > 0.0) ? powe(ax, pexp - 1.0, ie1) : 0.0;
    const double d = cdt * pw1 * x;
    dg[a] = d;
    kk[a] = cdt * pexp * pw1 * ig[a];
#pragma unroll
    for (int k = 0; k < 9; ++k) L[k] = fma(d, m.p9[a][k], L[k]);
  }
#pragma unroll
  for (int k = 0; k < 9; ++k) B[k] = ((k % 4) == 0 ? 1.0 : 0.0) - L[k];
  mm3(Ct, B, M);
  // E = (B^T M - I)/2 in 6-component form
  double e[6];
  e[0] = 0.5 * (fma(B[0], M[0], fma(B[3], M[3], B[6] * M[6])) - 1.0);
  e[1] = 0.5 * (fma(B[1], M[1], fma(B[4], M[4], B[7] * M[7])) - 1.0);
  e[2] = 0.5 * (fma(B[2], M[2], fma(B[5], M[5], B[8] * M[8])) - 1.0);
  e[3] = 0.5 * fma(B[1], M[2], fma(B[4], M[5], B[7] * M[8]));
  e[4] = 0.5 * fma(B[0], M[2], fma(B[3], M[5], B[6] * M[8]));
  e[5] = 0.5 * fma(B[0], M[1], fma(B[3], M[4], B[6] * M[7]));
  double t[6];
  cubic_apply(cc, e, t);
#pragma unroll
  for (int k = 0; k < 6; ++k) r[k] = s[k] - t[k];
  const double n2 = fma(r[0], r[0], fma(r[1], r[1], r[2] * r[2])) +
                    2.0 * fma(r[3], r[3], fma(r[4], r[4], r[5] * r[5]));
  rn = sqrt(n2);
}

// J = dr/ds = I + sum_a kk_a (C : sym(M^T d_a (x) n_a)) (x) pv_a
//           = I + C : Q,   Q = sum_a sym(M^T d_a (x) n_a) (x) (kk_a pv_a)
// (C is linear, so it is applied once to the six columns of Q instead of once per slip
// system).
template <int NS>
CPFEM_HD void cp_jacobian(const MatDev& m, const Cub& cc, const double* kk, const double* M,
                                            double* J) {
  double* Q = J;   // Q accumulates in J, then J = I + C : Q column by column in place
#pragma unroll
  for (int i = 0; i < 36; ++i) Q[i] = 0.0;
#pragma unroll
  for (int a = 0; a < NS; ++a) {
    const double* d = m.d[a];
    const double* n = m.n[a];
    double w[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) w[i] = fma(M[i], d[0], fma(M[3 + i], d[1], M[6 + i] * d[2]));
    double q[6];
    q[0] = w[0] * n[0];
    q[1] = w[1] * n[1];
    q[2] = w[2] * n[2];
    q[3] = 0.5 * fma(w[1], n[2], w[2] * n[1]);
    q[4] = 0.5 * fma(w[0], n[2], w[2] * n[0]);
    q[5] = 0.5 * fma(w[0], n[1], w[1] * n[0]);
    double c[6];
#pragma unroll
    for (int j = 0; j < 6; ++j) c[j] = kk[a] * m.pv[a][j];
#pragma unroll
    for (int i = 0; i < 6; ++i)
#pragma unroll
      for (int j = 0; j < 6; ++j) Q[6 * i + j] = fma(q[i], c[j], Q[6 * i + j]);
  }
#pragma unroll
  for (int j = 0; j < 6; ++j) {
    double col[6], t[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) col[i] = Q[6 * i + j];
    cubic_apply(cc, col, t);
#pragma unroll
    for (int i = 0; i < 6; ++i) J[6 * i + j] = (i == j ? 1.0 : 0.0) + t[i];
  }
}

// The same Jacobian in FP32, for a Newton direction only (the residual, the stop test and
// the tangent stay FP64).  Used while the Jacobian's scale max_a kk_a C11 is at most
// kJ32Scale, where FP32 rounding leaves the direction accurate to ~1e-4 or better.
constexpr double kJ32Scale = 1e4;

template <int NS>
CPFEM_HD void cp_jacobian_f32(const MatDev& m, const Cub& cc, const double* kk, const double* M, float* J) {
  float Mf[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) Mf[k] = f32_of(M[k]);
  float* Q = J;
#pragma unroll
  for (int i = 0; i < 36; ++i) Q[i] = 0.0f;
#pragma unroll
  for (int a = 0; a < NS; ++a) {
    const float* d = m.d32[a];
    const float* n = m.n32[a];
    float w[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) w[i] = fmaf(Mf[i], d[0], fmaf(Mf[3 + i], d[1], Mf[6 + i] * d[2]));
    float q[6];
    q[0] = w[0] * n[0];
    q[1] = w[1] * n[1];
    q[2] = w[2] * n[2];
    q[3] = 0.5f * fmaf(w[1], n[2], w[2] * n[1]);
    q[4] = 0.5f * fmaf(w[0], n[2], w[2] * n[0]);
    q[5] = 0.5f * fmaf(w[0], n[1], w[1] * n[0]);
    const float ka = f32_of(kk[a]);
    float c[6];
#pragma unroll
    for (int j = 0; j < 6; ++j) c[j] = ka * m.pv32[a][j];
#pragma unroll
    for (int i = 0; i < 6; ++i)
#pragma unroll
      for (int j = 0; j < 6; ++j) Q[6 * i + j] = fmaf(q[i], c[j], Q[6 * i + j]);
  }
  const float c11 = f32_of(cc.C11), c12 = f32_of(cc.C12), c44x2 = f32_of(2.0 * cc.C44);
#pragma unroll
  for (int j = 0; j < 6; ++j) {
    const float e0 = Q[j], e1 = Q[6 + j], e2 = Q[12 + j];
    const float t0 = fmaf(c11, e0, c12 * (e1 + e2));
    const float t1 = fmaf(c11, e1, c12 * (e0 + e2));
    const float t2 = fmaf(c11, e2, c12 * (e0 + e1));
    J[j] = (j == 0 ? 1.0f : 0.0f) + t0;
    J[6 + j] = (j == 1 ? 1.0f : 0.0f) + t1;
    J[12 + j] = (j == 2 ? 1.0f : 0.0f) + t2;
#pragma unroll
    for (int i = 3; i < 6; ++i) J[6 * i + j] = (i == j ? 1.0f : 0.0f) + c44x2 * Q[6 * i + j];
  }
}

// The FP64 Newton direction of the local solve, ds = -J^-1 r (the reference's).
template <int NS>
CPFEM_HD void cp_direction_f64(const MatDev& m, const Cub& cc, const double* kk, const double* M, const double* r,
                               double* ds) {
  double J[36];
  int perm[6];
  double dinv[6];
  cp_jacobian<NS>(m, cc, kk, M, J);
  lu_factor<6>(J, perm, dinv);
#pragma unroll
  for (int k = 0; k < 6; ++k) ds[k] = -r[k];
  lu_solve<6>(J, perm, dinv, ds);
}

template <int NS>
struct DirIn {
  double kk[NS];
  double M[9];
  double r[6];
};
struct Vec6 {
  double v[6];
};

#ifdef __CUDACC__
template <int NS>
__device__ __noinline__ Vec6 cp_direction_f64_cold(const MatDev& m, Cub cc, DirIn<NS> in) {
  Vec6 o;
  cp_direction_f64<NS>(m, cc, in.kk, in.M, in.r, o.v);
  return o;
}
#endif

constexpr int kWarmStartIters = 8;   // a warm start still unconverged after this restarts from 0

// Local Newton with the cut-half line search of models_copper.py:218-245: trial
// residuals at s + relax ds, relax = 1, 1/2, ..., until the norm drops below the current
// one or max_sub_step trials were made; the last trial is taken.  It starts from s0 = 0,
// as the reference does, or -- given s_init, the same GP's last converged stress -- from
// there, which needs far fewer iterations once the global Newton iterates settle.  A
// warm start that has not converged after kWarmStartIters iterations (or went
// non-finite) is abandoned: one step with a single trial evaluates the residual at
// s0 = 0 and the reference's iteration runs from there with its own max_iter.  Either way the result is the root of the same residual to the
// same tolerance.  st.iters counts every step, the restart included.
template <int NS>
CPFEM_HD void cp_local_newton(const MatDev& m, const Cub& cc, const double* Ct, const double* ig,
                                                double cdt, double pexp, GPSolve<NS>& st,
                                                const double* s_init = nullptr, bool j32 = false) {
  const int ie1 = int_exponent(pexp - 1.0);
  double r[6];
  bool warm = s_init != nullptr;
#pragma unroll
  for (int k = 0; k < 6; ++k) st.s[k] = warm ? s_init[k] : 0.0;
  cp_residual<NS>(m, cc, Ct, ig, cdt, pexp, ie1, st.s, r, st.rn, st.dg, st.kk, st.B, st.M);
  const int warm_iters = (kWarmStartIters < m.max_iter) ? kWarmStartIters : m.max_iter - 1;
  int it = 0, it0 = 0;   // it0: the step the s0 = 0 iteration started at
  while ((st.rn > m.local_tol || (warm && !(st.rn <= m.local_tol))) && it - it0 < m.max_iter) {
    double ds[6];
    int sub_cap = m.max_sub_step;
    if (warm && (it >= warm_iters || !isfinite(st.rn))) {
      // abandon the warm start: the single trial below lands on s = 0 + 1 * 0
#pragma unroll
      for (int k = 0; k < 6; ++k) st.s[k] = ds[k] = 0.0;
      sub_cap = 1;
      warm = false;
      it0 = it + 1;
    } else {
      bool done = false;
      if (j32) {
        double kmax = 0.0;
#pragma unroll
        for (int a = 0; a < NS; ++a) kmax = fmax(kmax, st.kk[a]);
        if (kmax * cc.C11 <= kJ32Scale) {
          float J[36], dinv[6], d32[6];
          int perm[6];
          cp_jacobian_f32<NS>(m, cc, st.kk, st.M, J);
          lu_factor<6>(J, perm, dinv);
#pragma unroll
          for (int k = 0; k < 6; ++k) d32[k] = -f32_of(r[k]);
          lu_solve<6>(J, perm, dinv, d32);
          done = true;
#pragma unroll
          for (int k = 0; k < 6; ++k) {
            ds[k] = f64_of(d32[k]);
            done = done && isfinite(ds[k]);
          }
        }
      }
      if (!done) {
#ifdef __CUDA_ARCH__
        if (j32) {
          // the cold path of FP32 directions: out of line, so its code and registers stay
          // out of the hot loop (inputs and result by value: no local array escapes)
          DirIn<NS> in;
#pragma unroll
          for (int a = 0; a < NS; ++a) in.kk[a] = st.kk[a];
#pragma unroll
          for (int k = 0; k < 9; ++k) in.M[k] = st.M[k];
#pragma unroll
          for (int k = 0; k < 6; ++k) in.r[k] = r[k];
          const Vec6 d = cp_direction_f64_cold<NS>(m, cc, in);
#pragma unroll
          for (int k = 0; k < 6; ++k) ds[k] = d.v[k];
        } else
#endif
        {
          cp_direction_f64<NS>(m, cc, st.kk, st.M, r, ds);
        }
      }
    }
    const double rn0 = sub_cap == 1 ? 0.0 : st.rn;
    double relax = 1.0;
    int sub = 0;
    double st_s[6];
    do {
#pragma unroll
      for (int k = 0; k < 6; ++k) st_s[k] = fma(relax, ds[k], st.s[k]);
      cp_residual<NS>(m, cc, Ct, ig, cdt, pexp, ie1, st_s, r, st.rn, st.dg, st.kk, st.B, st.M);
      relax *= 0.5;
      ++sub;
    } while (st.rn >= rn0 && sub < sub_cap);
    // s + 2 relax ds with the halved relax is exactly the last trial point
#pragma unroll
    for (int k = 0; k < 6; ++k) st.s[k] = st_s[k];
    ++it;
  }
  st.iters = it;
}

// Stress at the converged state.
//   H = Fp^-1_old R B,  Fe_l = F H,  P = F Y,  Y = H s H^T / det H
// (algebraically the reference's det(F) sigma F^-T with sigma = Fe S Fe^T / det Fe,
// models_copper.py:155-162).  W = s H^T and 1/det H are kept for the tangent.
template <int NS>
CPFEM_HD void cp_stress(const double* F, const double* G /*Fp^-1_old R*/, const GPSolve<NS>& st, double* H,
                        double* W, double* Y, double& idet, double* P) {
  double S[9];
  mm3(G, st.B, H);
  S[0] = st.s[0]; S[4] = st.s[1]; S[8] = st.s[2];
  S[5] = S[7] = st.s[3];
  S[2] = S[6] = st.s[4];
  S[1] = S[3] = st.s[5];
  idet = 1.0 / det3(H);
  mm3_bt(S, H, W);           // W = s H^T
  mm3(H, W, Y);              // H s H^T
#pragma unroll
  for (int k = 0; k < 9; ++k) Y[k] *= idet;
  mm3(F, Y, P);
}

// Slip tables in the precision of a tangent computation.
CPFEM_HD double tan_p9(const MatDev& m, double, int a, int k) { return m.p9[a][k]; }
CPFEM_HD float tan_p9(const MatDev& m, float, int a, int k) { return m.d32[a][k / 3] * m.n32[a][k % 3]; }
CPFEM_HD double tan_pv(const MatDev& m, double, int a, int j) { return m.pv[a][j]; }
CPFEM_HD float tan_pv(const MatDev& m, float, int a, int j) { return m.pv32[a][j]; }

template <int NS>
CPFEM_HD void tan_jacobian(const MatDev& m, const Cub& cc, const double* kk, const double* M, double* J) {
  cp_jacobian<NS>(m, cc, kk, M, J);
}
template <int NS>
CPFEM_HD void tan_jacobian(const MatDev& m, const Cub& cc, const double* kk, const double* M, float* J) {
  cp_jacobian_f32<NS>(m, cc, kk, M, J);
}

// Consistent tangent at the converged state:
// dP/dF = d_ik Y_lJ + (dP/ds)(ds/dF) with ds/dF = J^-1 C : sym(Fe_l[k,:] (x) H[l,:]),
// the implicit-function tangent of f_jvp (models_copper.py:251-259).
// The tangent column for F_kl is handed to store_col(kl, col[9], ds/dF_kl[6]), both in
// the precision T, as soon as it is known, so the 81 entries never need to be live at once.  Called after every other
// output of the Gauss point is written, so only what it needs is live.
// T is the precision of the computation: FP64, or FP32 for a tangent that only serves as
// the global Newton's Jacobian and the local solve's start prediction (the converged
// state and stress, and the residual that decides convergence, stay FP64 either way).
template <int NS, typename T, class StoreCol>
CPFEM_HD void cp_tangent_t(const MatDev& m, const Cub& cc, const double* F64, const double* G64,
                           const GPSolve<NS>& st, const double* H64, const double* W64, const double* Y64,
                           double idet64, StoreCol store_col) {
  T F[9], G[9], H[9], W[9], Y[9], B[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    F[k] = to_prec<T>(F64[k]); G[k] = to_prec<T>(G64[k]); H[k] = to_prec<T>(H64[k]);
    W[k] = to_prec<T>(W64[k]); Y[k] = to_prec<T>(Y64[k]); B[k] = to_prec<T>(st.B[k]);
  }
  const T idet = to_prec<T>(idet64);
  T kkT[NS];
#pragma unroll
  for (int a = 0; a < NS; ++a) kkT[a] = to_prec<T>(st.kk[a]);
  // dP/ds for the 6 symmetric basis directions
  T Bi[9];
  inv3(B, Bi);
  T dPds[6][9];
#pragma unroll
  for (int mm = 0; mm < 6; ++mm) {
    T dL[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) dL[k] = T(0);
#pragma unroll
    for (int a = 0; a < NS; ++a) {
      const T c = kkT[a] * tan_pv(m, T(0), a, mm);
#pragma unroll
      for (int k = 0; k < 9; ++k) dL[k] = cp_fma(c, tan_p9(m, T(0), a, k), dL[k]);
    }
    T trace = T(0);
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) trace = cp_fma(Bi[3 * i + j], dL[3 * j + i], trace);
    T dH[9], V[9], dY[9];
    mm3(G, dL, dH);          // G dL  (= -dH)
    mm3(dH, W, V);           // V = (G dL) s H^T
    const int ei = (mm < 3) ? mm : ((mm == 3) ? 1 : 0);
    const int ej = (mm < 3) ? mm : ((mm == 5) ? 1 : 2);
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        T hh = H[3 * i + ei] * H[3 * j + ej];
        if (mm >= 3) hh = cp_fma(H[3 * i + ej], H[3 * j + ei], hh);
        dY[3 * i + j] = cp_fma(hh - V[3 * i + j] - V[3 * j + i], idet, Y[3 * i + j] * trace);
      }
    mm3(F, dY, dPds[mm]);
  }

  // ds/dF column by column through the factorised Jacobian at the converged s
  T J[36];
  int perm[6];
  T dinv[6];
  tan_jacobian<NS>(m, cc, st.kk, st.M, J);
  lu_factor<6>(J, perm, dinv);
  T Fe[9];
  mm3(F, H, Fe);
#pragma unroll
  for (int kl = 0; kl < 9; ++kl) {
    const int k = kl / 3, l = kl % 3;
    T a[3], b[3];
#pragma unroll
    for (int t = 0; t < 3; ++t) {
      a[t] = Fe[3 * k + t];
      b[t] = H[3 * l + t];
    }
    T q[6], x[6];
    q[0] = a[0] * b[0];
    q[1] = a[1] * b[1];
    q[2] = a[2] * b[2];
    q[3] = T(0.5) * cp_fma(a[1], b[2], a[2] * b[1]);
    q[4] = T(0.5) * cp_fma(a[0], b[2], a[2] * b[0]);
    q[5] = T(0.5) * cp_fma(a[0], b[1], a[1] * b[0]);
    cubic_apply(cc, q, x);
    lu_solve<6>(J, perm, dinv, x);
    T col[9];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        T v = (i == k) ? Y[3 * l + j] : T(0);
#pragma unroll
        for (int mm = 0; mm < 6; ++mm) v = cp_fma(dPds[mm][3 * i + j], x[mm], v);
        col[3 * i + j] = v;
      }
    store_col(kl, col, x);
  }
}

template <int NS, class StoreCol>
CPFEM_HD void cp_tangent(const MatDev& m, const Cub& cc, const double* F, const double* G, const GPSolve<NS>& st,
                         const double* H, const double* W, const double* Y, double idet, StoreCol store_col) {
  cp_tangent_t<NS, double>(m, cc, F, G, st, H, W, Y, idet, store_col);
}

// The FP32 tangent is used while the local Jacobian's scale max_a kk_a C11 is at most
// kJ32Scale (as for the FP32 local directions), where its rounding leaves the tangent
// accurate to ~1e-4 relative or better; stiffer points get the FP64 one.
template <int NS>
CPFEM_HD bool tangent_f32_ok(const GPSolve<NS>& st, const Cub& cc) {
  double kmax = 0.0;
#pragma unroll
  for (int a = 0; a < NS; ++a) kmax = fmax(kmax, st.kk[a]);
  return kmax * cc.C11 <= kJ32Scale;
}

// Explicit hardening and slip update after the local solve (models_copper.py:176-187;
// per-GP parameters as in crystal_plasticity_OR_design/models_sens_rot.py:168-193).
template <int NS>
CPFEM_HD void cp_hardening(const MatDev& m, const double* g, const double* dg,
                                             double h, double t_sat, double gss_a, double rq,
                                             double* g_new) {
  double tmp[NS];
  double total = 0.0;
  const int ia = int_exponent(gss_a);
#pragma unroll
  for (int b = 0; b < NS; ++b) {
    const double ratio = 1.0 - g[b] / t_sat;
    const double ar = fabs(ratio);
    const double pw = (ar > 0.0) ? powe(ar, gss_a, ia) : 0.0;
    const double sg = (ratio > 0.0) ? 1.0 : ((ratio < 0.0) ? -1.0 : 0.0);
    tmp[b] = h * fabs(dg[b]) * pw * sg;
    total += tmp[b];
  }
  if (m.qmode == 0) {
#pragma unroll
    for (int a = 0; a < NS; ++a) g_new[a] = fma(rq, total, g[a]);
  } else {
#pragma unroll
    for (int a0 = 0; a0 < NS; a0 += 3) {
      const double blk = tmp[a0] + tmp[a0 + 1] + tmp[a0 + 2];
      const double inc = fma(rq, total - blk, blk);
#pragma unroll
      for (int j = 0; j < 3; ++j) g_new[a0 + j] = g[a0 + j] + inc;
    }
  }
}

}  // namespace cpfem
