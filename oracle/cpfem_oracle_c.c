/* CPU FP64 oracle, compiled part -- TEST INFRASTRUCTURE, NOT PRODUCT CODE.
 *
 * A plain C (OpenMP) restatement of the same algorithm as oracle/cpfem_oracle.py, for
 * the sizes where numpy is too slow: the 32^3 and 64^3 load steps that the parity tests
 * and the timed CPU baseline run end to end.  It follows the numpy oracle line by line
 * (same unknowns, same iteration, same order of decisions), and is checked against it
 * on small cases by the CPU test suite; the numpy oracle is in turn pinned to the
 * reference's golden curves.  Reference lines (paths relative to the reference project):
 *
 *   orc_gp_pass       singlecrystal_copper/models_copper.py:155-259 -- the S-based local
 *                     Newton on the 9 components of S in the global frame, cut-half line
 *                     search with the 2*relax update (:204-249), linearised Fp^-1 update
 *                     (:188-191), explicit Kalidindi hardening with the source-system
 *                     saturation (:176-187), the implicit-function tangent of f_jvp
 *                     (:251-259), P and sigma (:155-162, :297-319);
 *                     crystal_plasticity_OR_design/models_sens_rot.py:143-259 for the
 *                     per-GP parameters (gss_a, h, t_sat, xm, r).
 *   orc_element       the HEX8 / 2x2x2 Gauss element residual int P:grad v and its
 *                     tangent (JAX-FEM's kernels, called at
 *                     crystal_plasticity_OR_design/solver.py:392), from FE first principles.
 *   orc_gather        COO -> CSR with summed duplicates (solver.py:279-282).
 *   orc_zero_rows     PETSc zeroRows: Dirichlet rows become unit rows (solver.py:290-293).
 *   orc_bicgstab      jax.scipy.sparse.linalg.bicgstab with the Jacobi preconditioner,
 *                     tol = atol = 1e-10 (solver.py:19-48), same recurrences and stop
 *                     rule as the numpy restatement ``cpfem_oracle.bicgstab``.
 *
 * Only the test suite, __graft_entry__.smoke() and the CPU legs of bench.py load it.
 * Deterministic for a given thread count: every Gauss point and matrix row is computed
 * independently, and dot products are summed per thread in a fixed partition, then in
 * thread order.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define MAXN 24

int orc_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void orc_set_threads(int n)
{
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

static inline double sgn(double x) { return (x > 0.0) - (x < 0.0); }

static inline void mm3(const double *a, const double *b, double *c)   /* c = a b */
{
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            c[3 * i + j] = a[3 * i] * b[j] + a[3 * i + 1] * b[3 + j] + a[3 * i + 2] * b[6 + j];
}

static inline double det3(const double *a)
{
    return a[0] * (a[4] * a[8] - a[5] * a[7]) - a[1] * (a[3] * a[8] - a[5] * a[6]) +
           a[2] * (a[3] * a[7] - a[4] * a[6]);
}

static inline void inv3(const double *a, double *r)
{
    double d = det3(a);
    r[0] = (a[4] * a[8] - a[5] * a[7]) / d;
    r[1] = (a[2] * a[7] - a[1] * a[8]) / d;
    r[2] = (a[1] * a[5] - a[2] * a[4]) / d;
    r[3] = (a[5] * a[6] - a[3] * a[8]) / d;
    r[4] = (a[0] * a[8] - a[2] * a[6]) / d;
    r[5] = (a[2] * a[3] - a[0] * a[5]) / d;
    r[6] = (a[3] * a[7] - a[4] * a[6]) / d;
    r[7] = (a[1] * a[6] - a[0] * a[7]) / d;
    r[8] = (a[0] * a[4] - a[1] * a[3]) / d;
}

/* LU with partial pivoting of the n x n row-major a (in place); 0 on success. */
static int lu(double *a, int n, int *piv)
{
    for (int k = 0; k < n; ++k) {
        int p = k;
        double m = fabs(a[k * n + k]);
        for (int i = k + 1; i < n; ++i)
            if (fabs(a[i * n + k]) > m) { m = fabs(a[i * n + k]); p = i; }
        piv[k] = p;
        if (m == 0.0) return 1;
        if (p != k)
            for (int j = 0; j < n; ++j) { double t = a[k * n + j]; a[k * n + j] = a[p * n + j]; a[p * n + j] = t; }
        double inv = 1.0 / a[k * n + k];
        for (int i = k + 1; i < n; ++i) {
            double f = a[i * n + k] * inv;
            a[i * n + k] = f;
            for (int j = k + 1; j < n; ++j) a[i * n + j] -= f * a[k * n + j];
        }
    }
    return 0;
}

/* Solve with the factors of lu() for nrhs right-hand sides stored as columns of the
 * n x nrhs row-major b (in place). */
static void lu_solve(const double *a, int n, const int *piv, double *b, int nrhs)
{
    for (int k = 0; k < n; ++k)
        if (piv[k] != k)
            for (int c = 0; c < nrhs; ++c) { double t = b[k * nrhs + c]; b[k * nrhs + c] = b[piv[k] * nrhs + c]; b[piv[k] * nrhs + c] = t; }
    for (int i = 1; i < n; ++i)
        for (int k = 0; k < i; ++k) {
            double f = a[i * n + k];
            for (int c = 0; c < nrhs; ++c) b[i * nrhs + c] -= f * b[k * nrhs + c];
        }
    for (int i = n - 1; i >= 0; --i) {
        for (int k = i + 1; k < n; ++k) {
            double f = a[i * n + k];
            for (int c = 0; c < nrhs; ++c) b[i * nrhs + c] -= f * b[k * nrhs + c];
        }
        double inv = 1.0 / a[i * n + i];
        for (int c = 0; c < nrhs; ++c) b[i * nrhs + c] *= inv;
    }
}

/* ------------------------------------------------------------------------------------
 * One Gauss point's local problem (cpfem_oracle.GPBatch for one lane)
 * ---------------------------------------------------------------------------------- */
typedef struct {
    const double *F, *Fpi, *g, *Pr, *Cr;
    double A[9];        /* F Fp^-1_old */
    double coef, p;     /* ao dt, 1/m */
    int N;
} gp_t;

/* tau, Delta gamma and d(Delta gamma)/d tau (models_copper.py:173-174) */
static void slip_increment(const gp_t *b, const double *S, double *tau, double *dgam, double *kd)
{
    for (int a = 0; a < b->N; ++a) {
        const double *P = b->Pr + 9 * a;
        double t = 0.0;
        for (int k = 0; k < 9; ++k) t += S[k] * P[k];
        double x = t / b->g[a];
        double ax = fabs(x);
        tau[a] = t;
        dgam[a] = b->coef * pow(ax, b->p) * sgn(t);
        if (kd) kd[a] = ax > 0.0 ? b->coef * b->p * pow(ax, b->p - 1.0) / b->g[a] * sgn(x) * sgn(t) : 0.0;
    }
}

/* L_p increment, Fp^-1 (I - L) and Fe = F Fp^-1_new (models_copper.py:188-191) */
static void kinematics(const gp_t *b, const double *dgam, double *Fpi_new, double *Fe)
{
    double IL[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    for (int a = 0; a < b->N; ++a)
        for (int k = 0; k < 9; ++k) IL[k] -= dgam[a] * b->Pr[9 * a + k];
    mm3(b->Fpi, IL, Fpi_new);
    mm3(b->F, Fpi_new, Fe);
}

/* r(S) = S - C' : (Fe^T Fe - I)/2 (models_copper.py:195-201) */
static void residual(const gp_t *b, const double *S, double *r)
{
    double tau[MAXN], dgam[MAXN], Fpi_new[9], Fe[9], E[9];
    slip_increment(b, S, tau, dgam, NULL);
    kinematics(b, dgam, Fpi_new, Fe);
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            E[3 * i + j] = 0.5 * (Fe[i] * Fe[j] + Fe[3 + i] * Fe[3 + j] + Fe[6 + i] * Fe[6 + j] - (i == j));
    for (int ij = 0; ij < 9; ++ij) {
        double s = 0.0;
        for (int kl = 0; kl < 9; ++kl) s += b->Cr[9 * ij + kl] * E[kl];
        r[ij] = S[ij] - s;
    }
}

static double norm9(const double *r)
{
    double s = 0.0;
    for (int k = 0; k < 9; ++k) s += r[k] * r[k];
    return sqrt(s);
}

/* dr/dS (9x9 row-major), what jax.jacfwd evaluates at models_copper.py:226:
 * J = I - C' : sum_a kd_a sym(Fe^T dFe/dgamma_a) (x) P_a, with dFe/dgamma_a = -A P_a. */
static void jacobian(const gp_t *b, const double *S, double *J)
{
    double tau[MAXN], dgam[MAXN], kd[MAXN], Fpi_new[9], Fe[9], B[9], Q[81];
    slip_increment(b, S, tau, dgam, kd);
    kinematics(b, dgam, Fpi_new, Fe);
    /* B = Fe^T A */
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            B[3 * i + j] = Fe[i] * b->A[j] + Fe[3 + i] * b->A[3 + j] + Fe[6 + i] * b->A[6 + j];
    memset(Q, 0, sizeof(Q));
    for (int a = 0; a < b->N; ++a) {
        if (kd[a] == 0.0) continue;
        const double *P = b->Pr + 9 * a;
        double M[9], Ns[9];
        mm3(B, P, M);                                   /* Fe^T A P_a = -Fe^T dFe_a */
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) Ns[3 * i + j] = -0.5 * (M[3 * i + j] + M[3 * j + i]);
        for (int mn = 0; mn < 9; ++mn) {
            double f = kd[a] * Ns[mn];
            for (int kl = 0; kl < 9; ++kl) Q[9 * mn + kl] += f * P[kl];
        }
    }
    for (int ij = 0; ij < 9; ++ij)
        for (int kl = 0; kl < 9; ++kl) {
            double s = 0.0;
            for (int mn = 0; mn < 9; ++mn) s += b->Cr[9 * ij + mn] * Q[9 * mn + kl];
            J[9 * ij + kl] = (ij == kl) - s;
        }
}

/* Local Newton from y0 = 0 with the cut-half line search (models_copper.py:204-249).
 * Returns the iteration count, or -1 when max_it is reached unconverged. */
static int local_newton(const gp_t *b, double tol, int max_sub_step, int max_it, double *y)
{
    double r[9], J[81], dy[9], yt[9], rt[9];
    int piv[9];
    memset(y, 0, 9 * sizeof(double));
    residual(b, y, r);
    double rn = norm9(r);
    int its = 0;
    while (rn > tol) {
        if (its >= max_it) return -1;
        jacobian(b, y, J);
        for (int k = 0; k < 9; ++k) dy[k] = -r[k];
        if (lu(J, 9, piv)) return -1;
        lu_solve(J, 9, piv, dy, 1);
        double relax = 1.0, rn_try = rn;
        int sub = 0;
        memcpy(rt, r, sizeof(rt));
        while (rn_try >= rn && sub < max_sub_step) {
            for (int k = 0; k < 9; ++k) yt[k] = y[k] + relax * dy[k];
            residual(b, yt, rt);
            rn_try = norm9(rt);
            relax *= 0.5;
            sub += 1;
        }
        for (int k = 0; k < 9; ++k) y[k] = y[k] + 2.0 * relax * dy[k];
        memcpy(r, rt, sizeof(r));
        rn = rn_try;
        its += 1;
        if (!(rn == rn)) return -1;
    }
    return its;
}

/* sigma = Fe S Fe^T / det Fe ; P = det F sigma F^-T (models_copper.py:155-162) */
static void first_pk(const gp_t *b, const double *S, double *P)
{
    double tau[MAXN], dgam[MAXN], Fpi_new[9], Fe[9], T[9], sig[9], Fi[9];
    slip_increment(b, S, tau, dgam, NULL);
    kinematics(b, dgam, Fpi_new, Fe);
    double FeT[9] = {Fe[0], Fe[3], Fe[6], Fe[1], Fe[4], Fe[7], Fe[2], Fe[5], Fe[8]};
    mm3(Fe, S, T);
    mm3(T, FeT, sig);
    double dFe = det3(Fe), dF = det3(b->F);
    for (int k = 0; k < 9; ++k) sig[k] = dF * (sig[k] / dFe);
    inv3(b->F, Fi);
    double FiT[9] = {Fi[0], Fi[3], Fi[6], Fi[1], Fi[4], Fi[7], Fi[2], Fi[5], Fi[8]};
    mm3(sig, FiT, P);
}

/* Consistent tangent dP/dF (81, [ij][kl]) at the converged S via the implicit-function
 * theorem of f_jvp (models_copper.py:251-259), as cpfem_oracle.tangent writes it out. */
static int tangent(const gp_t *b, const double *S, double *D)
{
    double tau[MAXN], dgam[MAXN], kd[MAXN], Fpi_new[9], Fe[9];
    double drdF[81], J[81], X[9], T1[9], Fpn_T[9], Fpi_inv[9];
    int piv[9];
    slip_increment(b, S, tau, dgam, kd);
    kinematics(b, dgam, Fpi_new, Fe);
    /* dr/dF_kl = -C' : sym(Fe^T e_k e_l^T Fpi_new); (Fe^T e_k e_l^T Fpi)_mn = Fe_km Fpi_ln */
    for (int k = 0; k < 3; ++k)
        for (int l = 0; l < 3; ++l) {
            double Ts[9];
            for (int m = 0; m < 3; ++m)
                for (int n = 0; n < 3; ++n)
                    Ts[3 * m + n] = 0.5 * (Fe[3 * k + m] * Fpi_new[3 * l + n] + Fe[3 * k + n] * Fpi_new[3 * l + m]);
            for (int ij = 0; ij < 9; ++ij) {
                double s = 0.0;
                for (int mn = 0; mn < 9; ++mn) s += b->Cr[9 * ij + mn] * Ts[mn];
                drdF[9 * ij + 3 * k + l] = -s;
            }
        }
    jacobian(b, S, J);
    if (lu(J, 9, piv)) return 1;
    for (int k = 0; k < 81; ++k) drdF[k] = -drdF[k];
    lu_solve(J, 9, piv, drdF, 9);                       /* dS/dF, [ij][kl] */
    const double *dSdF = drdF;
    double detFpi = det3(Fpi_new);
    for (int k = 0; k < 9; ++k) Fpn_T[k] = Fpi_new[3 * (k % 3) + k / 3];
    mm3(Fpi_new, S, T1);
    mm3(T1, Fpn_T, X);
    for (int k = 0; k < 9; ++k) X[k] /= detFpi;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            for (int k = 0; k < 3; ++k)
                for (int l = 0; l < 3; ++l) D[27 * i + 9 * j + 3 * k + l] = (i == k) ? X[3 * l + j] : 0.0;
    inv3(Fpi_new, Fpi_inv);
    double dPdS[81];
    for (int m = 0; m < 3; ++m)
        for (int n = 0; n < 3; ++n) {
            double dL[9] = {0}, dFpi[9], t1[9], t2[9], t3[9], dX[9], tr = 0.0;
            for (int a = 0; a < b->N; ++a) {
                double f = kd[a] * b->Pr[9 * a + 3 * m + n];
                for (int k = 0; k < 9; ++k) dL[k] += f * b->Pr[9 * a + k];
            }
            mm3(b->Fpi, dL, dFpi);
            for (int k = 0; k < 9; ++k) dFpi[k] = -dFpi[k];
            double dFpi_T[9];
            for (int k = 0; k < 9; ++k) dFpi_T[k] = dFpi[3 * (k % 3) + k / 3];
            /* dFpi S Fpi^T + Fpi E_mn Fpi^T + Fpi S dFpi^T */
            mm3(dFpi, S, t1);
            mm3(t1, Fpn_T, t2);
            mm3(T1, dFpi_T, t3);
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j)
                    dX[3 * i + j] = (t2[3 * i + j] + Fpi_new[3 * i + m] * Fpi_new[3 * j + n] + t3[3 * i + j]) / detFpi;
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) tr += Fpi_inv[3 * i + j] * dFpi[3 * j + i];
            for (int k = 0; k < 9; ++k) dX[k] -= X[k] * tr;
            double FdX[9];
            mm3(b->F, dX, FdX);
            for (int ij = 0; ij < 9; ++ij) dPdS[9 * ij + 3 * m + n] = FdX[ij];
        }
    for (int ij = 0; ij < 9; ++ij)
        for (int kl = 0; kl < 9; ++kl) {
            double s = 0.0;
            for (int mn = 0; mn < 9; ++mn) s += dPdS[9 * ij + mn] * dSdF[9 * mn + kl];
            D[9 * ij + kl] += s;
        }
    return 0;
}

/* F = I + sum_a u_a (x) dN_a/dX at every GP (models_copper.py:277-278). */
void orc_deformation(long E, const long *cells, const double *sg, const double *u, double *F)
{
#pragma omp parallel for schedule(static)
    for (long e = 0; e < E; ++e)
        for (int q = 0; q < 8; ++q) {
            double *f = F + 9 * (8 * e + q);
            const double *s = sg + 24 * (8 * e + q);
            for (int k = 0; k < 9; ++k) f[k] = (k % 4 == 0) ? 1.0 : 0.0;
            for (int a = 0; a < 8; ++a) {
                const double *ua = u + 3 * cells[8 * e + a];
                for (int i = 0; i < 3; ++i)
                    for (int j = 0; j < 3; ++j) f[3 * i + j] += ua[i] * s[3 * a + j];
            }
        }
}

/* The constitutive pass over G Gauss points.  Per-GP inputs: F (9), Fpi (9), g (N),
 * slip (N), rotation index into Pr_tab (nrot, N, 9) / Cr_tab (nrot, 81), parameters
 * (G, 5) = (gss_a, h, t_sat, xm, r).  Outputs (each may be NULL): P (9), D (81), sigma
 * (9, Cauchy P F^T / det F), Fpi_new (9), g_new (N), slip_new (N), its.  Returns the
 * number of GPs whose local Newton did not converge within max_it. */
long orc_gp_pass(long G, int N, const double *F, const double *Fpi, const double *g, const double *slip,
                 const int *rot_idx, const double *Pr_tab, const double *Cr_tab, const double *params,
                 int coplanar, double ao, double dt, double tol, int max_sub_step, int max_it,
                 double *P, double *D, double *sigma, double *Fpi_new, double *g_new, double *slip_new, int *its)
{
    long bad = 0;
    if (N > MAXN) return G;
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : bad)
    for (long k = 0; k < G; ++k) {
        gp_t b;
        b.F = F + 9 * k;
        b.Fpi = Fpi + 9 * k;
        b.g = g + (long)N * k;
        b.Pr = Pr_tab + (long)9 * N * rot_idx[k];
        b.Cr = Cr_tab + 81L * rot_idx[k];
        b.N = N;
        const double *pr = params + 5 * k;
        b.coef = ao * dt;
        b.p = 1.0 / pr[3];
        mm3(b.F, b.Fpi, b.A);
        double S[9];
        int it = local_newton(&b, tol, max_sub_step, max_it, S);
        if (its) its[k] = it;
        if (it < 0) { bad += 1; continue; }
        double Pk[9];
        if (P || sigma) first_pk(&b, S, Pk);
        if (P) memcpy(P + 9 * k, Pk, sizeof(Pk));
        if (sigma) {
            const double *f = b.F;
            double FT[9] = {f[0], f[3], f[6], f[1], f[4], f[7], f[2], f[5], f[8]}, s[9];
            mm3(Pk, FT, s);
            double d = det3(f);
            for (int m = 0; m < 9; ++m) sigma[9 * k + m] = s[m] / d;
        }
        if (D && tangent(&b, S, D + 81 * k)) { bad += 1; continue; }
        if (Fpi_new || g_new || slip_new) {
            /* explicit state update (models_copper.py:176-187; per-GP parameters as
             * models_sens_rot.py:168-193); q = r with ones on the coplanar 3-blocks */
            double tau[MAXN], dgam[MAXN], fpn[9], Fe[9], tmp[MAXN];
            slip_increment(&b, S, tau, dgam, NULL);
            kinematics(&b, dgam, fpn, Fe);
            if (Fpi_new) memcpy(Fpi_new + 9 * k, fpn, sizeof(fpn));
            double gss_a = pr[0], h = pr[1], t_sat = pr[2], r = pr[4];
            for (int a = 0; a < N; ++a) {
                double ratio = 1.0 - b.g[a] / t_sat;
                tmp[a] = h * fabs(dgam[a]) * pow(fabs(ratio), gss_a) * sgn(ratio);
            }
            if (g_new)
                for (int i = 0; i < N; ++i) {
                    double s = 0.0;
                    for (int j = 0; j < N; ++j) {
                        double q = (coplanar && j / 3 == i / 3) ? 1.0 : r;
                        s += q * tmp[j];
                    }
                    g_new[(long)N * k + i] = b.g[i] + s;
                }
            if (slip_new)
                for (int a = 0; a < N; ++a) slip_new[(long)N * k + a] = slip[(long)N * k + a] + dgam[a];
        }
    }
    return bad;
}

/* Element residual (E, 24) and tangent (E, 24, 24) of the HEX8 / 2x2x2 Gauss element:
 * R_ai = sum_q P_iJ dN_a/dX_J JxW, K_(ai)(bk) = sum_q dN_a/dX_J dP_iJ/dF_kL dN_b/dX_L JxW. */
void orc_element(long E, const double *sg, const double *jxw, const double *P, const double *D,
                 double *re, double *ke)
{
#pragma omp parallel for schedule(static)
    for (long e = 0; e < E; ++e) {
        double *r = re + 24 * e;
        memset(r, 0, 24 * sizeof(double));
        double *K = ke ? ke + 576 * e : NULL;
        if (K) memset(K, 0, 576 * sizeof(double));
        for (int q = 0; q < 8; ++q) {
            long gp = 8 * e + q;
            const double *s = sg + 24 * gp, *p = P + 9 * gp;
            double w = jxw[gp];
            for (int a = 0; a < 8; ++a)
                for (int i = 0; i < 3; ++i)
                    r[3 * a + i] += (p[3 * i] * s[3 * a] + p[3 * i + 1] * s[3 * a + 1] + p[3 * i + 2] * s[3 * a + 2]) * w;
            if (!K) continue;
            const double *d = D + 81 * gp;
            double Gm[8][3][3][3];          /* sum_J dN_a/dX_J D_iJkL */
            for (int a = 0; a < 8; ++a)
                for (int i = 0; i < 3; ++i)
                    for (int k = 0; k < 3; ++k)
                        for (int l = 0; l < 3; ++l)
                            Gm[a][i][k][l] = s[3 * a] * d[27 * i + 3 * k + l] + s[3 * a + 1] * d[27 * i + 9 + 3 * k + l] +
                                             s[3 * a + 2] * d[27 * i + 18 + 3 * k + l];
            for (int a = 0; a < 8; ++a)
                for (int i = 0; i < 3; ++i)
                    for (int b2 = 0; b2 < 8; ++b2)
                        for (int k = 0; k < 3; ++k)
                            K[24 * (3 * a + i) + 3 * b2 + k] +=
                                (Gm[a][i][k][0] * s[3 * b2] + Gm[a][i][k][1] * s[3 * b2 + 1] + Gm[a][i][k][2] * s[3 * b2 + 2]) * w;
        }
    }
}

/* out[p] = sum over k in [ptr[p], ptr[p+1]) of src[idx[k]], in list order: the summed
 * duplicates of the element COO triplets, in element order. */
void orc_gather(long n, const long *ptr, const long *idx, const double *src, double *out)
{
#pragma omp parallel for schedule(static)
    for (long p = 0; p < n; ++p) {
        double s = 0.0;
        for (long k = ptr[p]; k < ptr[p + 1]; ++k) s += src[idx[k]];
        out[p] = s;
    }
}

/* PETSc zeroRows with the pattern kept: every listed row is zero but a unit diagonal. */
void orc_zero_rows(long nrows, const long *rows, const long *indptr, const int *indices, double *data)
{
#pragma omp parallel for schedule(static)
    for (long k = 0; k < nrows; ++k) {
        long r = rows[k];
        for (long j = indptr[r]; j < indptr[r + 1]; ++j) data[j] = (indices[j] == r) ? 1.0 : 0.0;
    }
}

/* y = A x (CSR) */
void orc_spmv(long n, const long *indptr, const int *indices, const double *data, const double *x, double *y)
{
#pragma omp parallel for schedule(static)
    for (long i = 0; i < n; ++i) {
        double s = 0.0;
        for (long j = indptr[i]; j < indptr[i + 1]; ++j) s += data[j] * x[indices[j]];
        y[i] = s;
    }
}

/* ------------------------------------------------------------------------------------
 * BiCGSTAB (jax.scipy.sparse.linalg.bicgstab, JAX 0.4.x) with M = diag(1/A_ii)
 * ---------------------------------------------------------------------------------- */
#define MAXT 1024

/* deterministic dot: fixed partition of [0, n) over nt parts, summed in part order */
static double pdot(long n, const double *a, const double *b, int nt, double *part)
{
#pragma omp parallel for schedule(static, 1) num_threads(nt)
    for (int t = 0; t < nt; ++t) {
        long lo = n * t / nt, hi = n * (t + 1) / nt;
        double s = 0.0;
        for (long i = lo; i < hi; ++i) s += a[i] * b[i];
        part[t] = s;
    }
    double s = 0.0;
    for (int t = 0; t < nt; ++t) s += part[t];
    return s;
}

/* Returns 0; *k_out = iterations, or -10 (rho = 0) / -11 (alpha or omega = 0) as jax. */
int orc_bicgstab(long n, const long *indptr, const int *indices, const double *data, const double *b, double *x,
                 const double *minv, double tol, double atol, int maxiter, int *k_out)
{
    int nt = orc_num_threads();
    if (nt > MAXT) nt = MAXT;
    double part[MAXT];
    double *r = malloc(8 * n * sizeof(double));
    if (!r) return 1;
    double *rhat = r + n, *p = r + 2 * n, *q = r + 3 * n, *phat = r + 4 * n, *s = r + 5 * n, *shat = r + 6 * n,
           *t = r + 7 * n;
    double bb = pdot(n, b, b, nt, part);
    double atol2 = tol * tol * bb > atol * atol ? tol * tol * bb : atol * atol;
    orc_spmv(n, indptr, indices, data, x, r);
#pragma omp parallel for schedule(static)
    for (long i = 0; i < n; ++i) {
        r[i] = b[i] - r[i];
        rhat[i] = p[i] = q[i] = r[i];
    }
    double rho = 1.0, alpha = 1.0, omega = 1.0;
    int k = 0;
    while (pdot(n, r, r, nt, part) > atol2 && k >= 0 && k < maxiter) {
        double rho_ = pdot(n, rhat, r, nt, part);
        double beta = rho_ / rho * alpha / omega;
#pragma omp parallel for schedule(static)
        for (long i = 0; i < n; ++i) {
            p[i] = r[i] + beta * (p[i] - omega * q[i]);
            phat[i] = p[i] * minv[i];
        }
        orc_spmv(n, indptr, indices, data, phat, q);
        alpha = rho_ / pdot(n, rhat, q, nt, part);
#pragma omp parallel for schedule(static)
        for (long i = 0; i < n; ++i) {
            s[i] = r[i] - alpha * q[i];
            shat[i] = s[i] * minv[i];
        }
        int exit_early = pdot(n, s, s, nt, part) < atol2;
        orc_spmv(n, indptr, indices, data, shat, t);
        omega = pdot(n, t, s, nt, part) / pdot(n, t, t, nt, part);
        if (exit_early) {
#pragma omp parallel for schedule(static)
            for (long i = 0; i < n; ++i) {
                x[i] = x[i] + alpha * phat[i];
                r[i] = s[i];
            }
        } else {
#pragma omp parallel for schedule(static)
            for (long i = 0; i < n; ++i) {
                x[i] = x[i] + (alpha * phat[i] + omega * shat[i]);
                r[i] = s[i] - omega * t[i];
            }
        }
        k = (omega == 0.0 || alpha == 0.0) ? -11 : k + 1;
        if (rho_ == 0.0) k = -10;
        rho = rho_;
    }
    free(r);
    *k_out = k;
    return 0;
}
