// Backward of the converged local Newton (the implicit-function VJP of the reference's
// custom_jvp, singlecrystal_copper/models_copper.py:251-259, as jax.grad transposes it).
//
// y(s, x) evaluates, at a fixed lattice-frame stress s, the residual r and the outputs
// (P, sigma, Fp^-1_new, g_new) from the inputs x = (F, Fp^-1_old, g, rotation, params).
// At the converged s (r = 0) a cotangent ybar on the outputs pulls back to
//   xbar = (dy/dx)^T ybar - (dr/dx)^T nu,   nu = J^-T (dy/ds)^T ybar,   J = dr/ds.
// The partial derivatives are taken in forward mode with K-tangent dual numbers over the
// same formulas as the forward pass, K directions per sweep.
#pragma once

#include "gp_update.cuh"

namespace cpfem {

template <int K>
struct Dual {
  double v;
  double d[K];
};

template <int K>
CPFEM_HD Dual<K> dconst(double v) {
  Dual<K> r;
  r.v = v;
#pragma unroll
  for (int k = 0; k < K; ++k) r.d[k] = 0.0;
  return r;
}

template <int K>
CPFEM_HD Dual<K> operator+(const Dual<K>& a, const Dual<K>& b) {
  Dual<K> r;
  r.v = a.v + b.v;
#pragma unroll
  for (int k = 0; k < K; ++k) r.d[k] = a.d[k] + b.d[k];
  return r;
}

template <int K>
CPFEM_HD Dual<K> operator-(const Dual<K>& a, const Dual<K>& b) {
  Dual<K> r;
  r.v = a.v - b.v;
#pragma unroll
  for (int k = 0; k < K; ++k) r.d[k] = a.d[k] - b.d[k];
  return r;
}

template <int K>
CPFEM_HD Dual<K> operator*(const Dual<K>& a, const Dual<K>& b) {
  Dual<K> r;
  r.v = a.v * b.v;
#pragma unroll
  for (int k = 0; k < K; ++k) r.d[k] = fma(a.d[k], b.v, a.v * b.d[k]);
  return r;
}

template <int K>
CPFEM_HD Dual<K> operator*(double a, const Dual<K>& b) {
  Dual<K> r;
  r.v = a * b.v;
#pragma unroll
  for (int k = 0; k < K; ++k) r.d[k] = a * b.d[k];
  return r;
}

template <int K>
CPFEM_HD Dual<K> recip(const Dual<K>& a) {
  Dual<K> r;
  r.v = 1.0 / a.v;
  const double c = -r.v * r.v;
#pragma unroll
  for (int k = 0; k < K; ++k) r.d[k] = c * a.d[k];
  return r;
}

// a*b + c
template <int K>
CPFEM_HD Dual<K> dfma(const Dual<K>& a, const Dual<K>& b, const Dual<K>& c) {
  Dual<K> r;
  r.v = fma(a.v, b.v, c.v);
#pragma unroll
  for (int k = 0; k < K; ++k) r.d[k] = fma(a.d[k], b.v, fma(a.v, b.d[k], c.d[k]));
  return r;
}

// sign(a) * a, derivative sign(a) (0 at a = 0, as jnp.abs differentiates)
template <int K>
CPFEM_HD Dual<K> dabs(const Dual<K>& a) {
  const double sg = (a.v > 0.0) ? 1.0 : ((a.v < 0.0) ? -1.0 : 0.0);
  return sg * a;
}

// x^q for x >= 0: value through powe, d = x^q (q dx/x + dq ln x); 0 at x = 0.
template <int K>
CPFEM_HD Dual<K> dpow(const Dual<K>& x, const Dual<K>& q, int iq) {
  Dual<K> r;
  if (x.v > 0.0) {
    r.v = powe(x.v, q.v, iq);
    const double a = r.v * q.v / x.v;
    const double lx = log(x.v);
#pragma unroll
    for (int k = 0; k < K; ++k) r.d[k] = fma(a, x.d[k], r.v * lx * q.d[k]);
  } else {
    r = dconst<K>(0.0);
  }
  return r;
}

template <int K>
CPFEM_HD void dmm3(const Dual<K>* A, const Dual<K>* B, Dual<K>* C) {
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j)
      C[3 * i + j] = dfma(A[3 * i], B[j], dfma(A[3 * i + 1], B[3 + j], A[3 * i + 2] * B[6 + j]));
}

template <int K>
CPFEM_HD void dmm3_bt(const Dual<K>* A, const Dual<K>* B, Dual<K>* C) {
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j)
      C[3 * i + j] = dfma(A[3 * i], B[3 * j], dfma(A[3 * i + 1], B[3 * j + 1], A[3 * i + 2] * B[3 * j + 2]));
}

template <int K>
CPFEM_HD void dmm3_at(const Dual<K>* A, const Dual<K>* B, Dual<K>* C) {
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j)
      C[3 * i + j] = dfma(A[i], B[j], dfma(A[3 + i], B[3 + j], A[6 + i] * B[6 + j]));
}

template <int K>
CPFEM_HD Dual<K> ddet3(const Dual<K>* A) {
  return A[0] * (A[4] * A[8] - A[5] * A[7]) - A[1] * (A[3] * A[8] - A[5] * A[6]) +
         A[2] * (A[3] * A[7] - A[4] * A[6]);
}

template <int K>
CPFEM_HD void dcubic(const Cub& m, const Dual<K>* e, Dual<K>* t) {
  t[0] = m.C11 * e[0] + m.C12 * (e[1] + e[2]);
  t[1] = m.C11 * e[1] + m.C12 * (e[0] + e[2]);
  t[2] = m.C11 * e[2] + m.C12 * (e[0] + e[1]);
  t[3] = (2.0 * m.C44) * e[3];
  t[4] = (2.0 * m.C44) * e[4];
  t[5] = (2.0 * m.C44) * e[5];
}

// Output block of y(s, x): residual r (6), P (9), sigma (9), Fp^-1_new (9), g_new (NS).
template <int NS>
struct YOut {
  static constexpr int kR = 0, kP = 6, kSig = 15, kFp = 24, kG = 33, kN = 33 + NS;
};

// Inputs of y(s, x): s (6), F (9), Fp^-1_old (9), g (NS), theta = (gss_a, h, t_sat, xm, rq) (5),
// w (3) -- a spatial rotation increment, R -> (I + [w]x) R, the only rotation directions
// on which the lattice-frame formulas and the reference's global-frame ones agree.
template <int NS>
struct XIn {
  static constexpr int kS = 0, kF = 6, kFp = 15, kG = 24, kTh = 24 + NS, kW = 29 + NS, kN = 32 + NS;
};

// One input value with its tangent seed: slot[idx] is the tangent slot of input idx, or -1.
template <int K>
CPFEM_HD Dual<K> seeded(const signed char* slot, int idx, double v) {
  Dual<K> r = dconst<K>(v);
  const int k = slot[idx];
#pragma unroll
  for (int j = 0; j < K; ++j) r.d[j] = (j == k) ? 1.0 : 0.0;
  return r;
}

// Evaluate y with dual tangents seeded by `slot` (XIn<NS>::kN entries).
// Returns the residual r (6 duals) and yb = sum_o ybar[o] y[o] over the output slots, so
// the outputs never have to be live at once.
template <int NS, int K>
CPFEM_HD void cp_eval_dual(const MatDev& m, const Cub& cc, double cdt, const double* s0, const double* F0,
                           const double* Fp0,
                           const double* g0, const double* R0, const double* th0, const signed char* slot,
                           const double* ybar, Dual<K>* r6, Dual<K>& yb) {
#define mk(idx, v) seeded<K>(slot, (idx), (v))
  Dual<K> s[6], F[9], Fp[9], R[9], th[5];
#pragma unroll
  for (int i = 0; i < 6; ++i) s[i] = mk(XIn<NS>::kS + i, s0[i]);
#pragma unroll
  for (int i = 0; i < 9; ++i) F[i] = mk(XIn<NS>::kF + i, F0[i]);
#pragma unroll
  for (int i = 0; i < 9; ++i) Fp[i] = mk(XIn<NS>::kFp + i, Fp0[i]);
#pragma unroll
  for (int i = 0; i < 5; ++i) th[i] = mk(XIn<NS>::kTh + i, th0[i]);
  {
    // R = (I + [w]x) R0 with w = 0 carrying the tangent
    Dual<K> w[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) w[i] = mk(XIn<NS>::kW + i, 0.0);
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const Dual<K> c0 = dconst<K>(R0[j]), c1 = dconst<K>(R0[3 + j]), c2 = dconst<K>(R0[6 + j]);
      // [w]x = [[0,-w2,w1],[w2,0,-w0],[-w1,w0,0]]
      R[j] = c0 + (c2 * w[1] - c1 * w[2]);
      R[3 + j] = c1 + (c0 * w[2] - c2 * w[0]);
      R[6 + j] = c2 + (c1 * w[0] - c0 * w[1]);
    }
  }
  Dual<K> A[9], AR[9], Ct[9];
  dmm3(F, Fp, A);
  dmm3(A, R, AR);
  dmm3_at(AR, AR, Ct);
  const Dual<K> pexp = recip(th[3]);
  const Dual<K> pm1 = pexp - dconst<K>(1.0);
  const int ie1 = int_exponent(pm1.v);
  const Dual<K> ga = th[0];
  const int ia = int_exponent(ga.v);
  Dual<K> L[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) L[k] = dconst<K>(0.0);
  Dual<K> tmp[NS];
  Dual<K> gv[NS];
#pragma unroll
  for (int a = 0; a < NS; ++a) {
    gv[a] = mk(XIn<NS>::kG + a, g0[a]);
    Dual<K> tau = dconst<K>(0.0);
#pragma unroll
    for (int c = 0; c < 6; ++c) tau = dfma(dconst<K>(m.pv[a][c]), s[c], tau);
    const Dual<K> x = tau * recip(gv[a]);
    const Dual<K> pw1 = dpow(dabs(x), pm1, ie1);
    const Dual<K> dg = cdt * (pw1 * x);
#pragma unroll
    for (int k = 0; k < 9; ++k) L[k] = dfma(dconst<K>(m.p9[a][k]), dg, L[k]);
    // hardening term of this system
    const Dual<K> ratio = dconst<K>(1.0) - gv[a] * recip(th[2]);
    const double sgn = (ratio.v > 0.0) ? 1.0 : ((ratio.v < 0.0) ? -1.0 : 0.0);
    tmp[a] = sgn * (th[1] * dabs(dg) * dpow(dabs(ratio), ga, ia));
  }
  Dual<K> B[9], M[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) B[k] = dconst<K>((k % 4 == 0) ? 1.0 : 0.0) - L[k];
  dmm3(Ct, B, M);
  Dual<K> e[6], t[6];
  e[0] = 0.5 * (dfma(B[0], M[0], dfma(B[3], M[3], B[6] * M[6])) - dconst<K>(1.0));
  e[1] = 0.5 * (dfma(B[1], M[1], dfma(B[4], M[4], B[7] * M[7])) - dconst<K>(1.0));
  e[2] = 0.5 * (dfma(B[2], M[2], dfma(B[5], M[5], B[8] * M[8])) - dconst<K>(1.0));
  e[3] = 0.5 * dfma(B[1], M[2], dfma(B[4], M[5], B[7] * M[8]));
  e[4] = 0.5 * dfma(B[0], M[2], dfma(B[3], M[5], B[6] * M[8]));
  e[5] = 0.5 * dfma(B[0], M[1], dfma(B[3], M[4], B[6] * M[7]));
  dcubic<K>(cc, e, t);
#pragma unroll
  for (int i = 0; i < 6; ++i) r6[i] = s[i] - t[i];
  yb = dconst<K>(0.0);
  // outputs
  Dual<K> G[9], H[9], S[9], W[9], Y[9];
  dmm3(Fp, R, G);
  dmm3(G, B, H);
  S[0] = s[0]; S[4] = s[1]; S[8] = s[2];
  S[5] = S[7] = s[3];
  S[2] = S[6] = s[4];
  S[1] = S[3] = s[5];
  const Dual<K> idet = recip(ddet3(H));
  dmm3_bt(S, H, W);
  dmm3(H, W, Y);
#pragma unroll
  for (int k = 0; k < 9; ++k) Y[k] = Y[k] * idet;
  Dual<K> P[9], sig[9], Fn[9];
  dmm3(F, Y, P);
  dmm3_bt(P, F, sig);
  const Dual<K> idf = recip(ddet3(F));
  dmm3_bt(H, R, Fn);
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    yb = dfma(dconst<K>(ybar[YOut<NS>::kP + k]), P[k], yb);
    yb = dfma(dconst<K>(ybar[YOut<NS>::kSig + k]), sig[k] * idf, yb);
    yb = dfma(dconst<K>(ybar[YOut<NS>::kFp + k]), Fn[k], yb);
  }
  Dual<K> total = dconst<K>(0.0);
#pragma unroll
  for (int a = 0; a < NS; ++a) total = total + tmp[a];
  const Dual<K> rq = th[4];
  if (m.qmode == 0) {
#pragma unroll
    for (int a = 0; a < NS; ++a) yb = dfma(dconst<K>(ybar[YOut<NS>::kG + a]), gv[a] + rq * total, yb);
  } else {
#pragma unroll
    for (int a0 = 0; a0 < NS; a0 += 3) {
      const Dual<K> blk = tmp[a0] + tmp[a0 + 1] + tmp[a0 + 2];
      const Dual<K> inc = rq * (total - blk) + blk;
#pragma unroll
      for (int j = 0; j < 3; ++j) yb = dfma(dconst<K>(ybar[YOut<NS>::kG + a0 + j]), gv[a0 + j] + inc, yb);
    }
  }
#undef mk
}

// Implicit-function VJP at the converged s.  ybar has YOut<NS>::kN entries (the residual
// slots are ignored); xbar receives the XIn<NS>::kN input cotangents for the directions
// listed in dirs[0..ndir) (others untouched).  Returns false if J is singular.
template <int NS, int K>
CPFEM_HD bool cp_vjp(const MatDev& m, const Cub& cc, double cdt, const double* s0, const double* F0,
                     const double* Fp0,
                     const double* g0, const double* R0, const double* th0, const double* ybar,
                     const int* dirs, int ndir, double* xbar) {
  // sweep 1: d/ds -> J (6x6) and sbar = (dy/ds)^T ybar
  constexpr int NX = XIn<NS>::kN;
  signed char slot[NX];
  double J[36], sbar[6];
  for (int c0 = 0; c0 < 6; c0 += K) {
    for (int i = 0; i < NX; ++i) slot[i] = (i >= c0 && i < c0 + K && i < 6) ? (signed char)(i - c0) : (signed char)-1;
    Dual<K> r6[6], yb;
    cp_eval_dual<NS, K>(m, cc, cdt, s0, F0, Fp0, g0, R0, th0, slot, ybar, r6, yb);
    for (int k = 0; k < K && c0 + k < 6; ++k) {
      for (int i = 0; i < 6; ++i) J[6 * i + c0 + k] = r6[i].d[k];
      sbar[c0 + k] = yb.d[k];
    }
  }
  // nu = J^-T sbar
  double JT[36];
  for (int i = 0; i < 6; ++i)
    for (int j = 0; j < 6; ++j) JT[6 * i + j] = J[6 * j + i];
  int perm[6];
  double dinv[6];
  lu_factor<6>(JT, perm, dinv);
  bool ok = true;
  for (int i = 0; i < 6; ++i) ok = ok && isfinite(dinv[i]);
  lu_solve<6>(JT, perm, dinv, sbar);
  // sweep 2: requested input directions
  for (int c0 = 0; c0 < ndir; c0 += K) {
    for (int i = 0; i < NX; ++i) slot[i] = -1;
    for (int k = 0; k < K && c0 + k < ndir; ++k) slot[dirs[c0 + k]] = (signed char)k;
    Dual<K> r6[6], yb;
    cp_eval_dual<NS, K>(m, cc, cdt, s0, F0, Fp0, g0, R0, th0, slot, ybar, r6, yb);
    for (int k = 0; k < K && c0 + k < ndir; ++k) {
      double acc = yb.d[k];
      for (int i = 0; i < 6; ++i) acc = fma(-sbar[i], r6[i].d[k], acc);
      xbar[dirs[c0 + k]] = acc;
    }
  }
  return ok;
}

}  // namespace cpfem
