// Shared helpers of the cpfem_gb300 CUDA sources: error reporting through the C ABI,
// the device-side material block and small fixed-size linear algebra in registers.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <string>

#include "../../include/cpfem_gb300.h"

// Small math helpers are host+device so the same code can be checked on the host.
#define CPFEM_HD __host__ __device__ __forceinline__

namespace cpfem {

// Thread-local text behind cpfem_last_error().
void set_error(const std::string& msg);

#define CPFEM_CUDA_TRY(expr)                                                              \
  do {                                                                                    \
    cudaError_t _e = (expr);                                                              \
    if (_e != cudaSuccess) {                                                              \
      ::cpfem::set_error(std::string(#expr) + ": " + cudaGetErrorString(_e));             \
      return CPFEM_ERR_CUDA;                                                              \
    }                                                                                     \
  } while (0)

#define CPFEM_REQUIRE(cond, msg)                                                          \
  do {                                                                                    \
    if (!(cond)) {                                                                        \
      ::cpfem::set_error(msg);                                                            \
      return CPFEM_ERR_ARG;                                                               \
    }                                                                                     \
  } while (0)

// Material block passed to kernels by value (it lands in the constant bank, so every
// warp reads it as a broadcast).  Built on the host from cpfem_material_t.
struct MatDev {
  int num_slip;
  int qmode;
  int max_sub_step;
  int max_iter;
  double local_tol;
  double ao;
  double C11, C12, C44;
  double d[CPFEM_MAX_SLIP][3];   // slip direction, lattice frame
  double n[CPFEM_MAX_SLIP][3];   // slip-plane normal, lattice frame
  double pv[CPFEM_MAX_SLIP][6];  // P = d n^T as (P11,P22,P33,P23+P32,P13+P31,P12+P21)
  double p9[CPFEM_MAX_SLIP][9];  // P = d n^T row-major
  float d32[CPFEM_MAX_SLIP][3];  // FP32 copies for the local Newton's FP32 direction
  float n32[CPFEM_MAX_SLIP][3];
  float pv32[CPFEM_MAX_SLIP][6];
};

int make_matdev(const cpfem_material_t* m, MatDev* out);

// Launch geometry shared by the vector kernels: a fixed grid keeps the reduction order
// (and so every dot product) identical from run to run.
constexpr int kVecThreads = 256;
constexpr int kVecBlocks = 2 * 152;

__host__ __device__ inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

// ---- 3x3 helpers (row-major) -------------------------------------------------------
CPFEM_HD void mm3(const double* A, const double* B, double* C) {
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j)
      C[3 * i + j] = fma(A[3 * i + 0], B[0 + j], fma(A[3 * i + 1], B[3 + j], A[3 * i + 2] * B[6 + j]));
}

// C = A * B^T
CPFEM_HD void mm3_bt(const double* A, const double* B, double* C) {
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j)
      C[3 * i + j] = fma(A[3 * i + 0], B[3 * j + 0], fma(A[3 * i + 1], B[3 * j + 1], A[3 * i + 2] * B[3 * j + 2]));
}

// C = A^T * B
CPFEM_HD void mm3_at(const double* A, const double* B, double* C) {
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j)
      C[3 * i + j] = fma(A[0 + i], B[0 + j], fma(A[3 + i], B[3 + j], A[6 + i] * B[6 + j]));
}

// FP32 versions of the 3x3 helpers, for the single-precision consistent tangent.
CPFEM_HD void mm3(const float* A, const float* B, float* C) {
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j)
      C[3 * i + j] = fmaf(A[3 * i + 0], B[0 + j], fmaf(A[3 * i + 1], B[3 + j], A[3 * i + 2] * B[6 + j]));
}

CPFEM_HD void inv3(const float* A, float* Ai) {
  const float c00 = A[4] * A[8] - A[5] * A[7];
  const float c01 = A[5] * A[6] - A[3] * A[8];
  const float c02 = A[3] * A[7] - A[4] * A[6];
  const float det = A[0] * c00 + A[1] * c01 + A[2] * c02;
  const float id = 1.0f / det;
  Ai[0] = c00 * id;
  Ai[1] = (A[2] * A[7] - A[1] * A[8]) * id;
  Ai[2] = (A[1] * A[5] - A[2] * A[4]) * id;
  Ai[3] = c01 * id;
  Ai[4] = (A[0] * A[8] - A[2] * A[6]) * id;
  Ai[5] = (A[2] * A[3] - A[0] * A[5]) * id;
  Ai[6] = c02 * id;
  Ai[7] = (A[1] * A[6] - A[0] * A[7]) * id;
  Ai[8] = (A[0] * A[4] - A[1] * A[3]) * id;
}

CPFEM_HD double det3(const double* A) {
  return A[0] * (A[4] * A[8] - A[5] * A[7]) - A[1] * (A[3] * A[8] - A[5] * A[6]) +
         A[2] * (A[3] * A[7] - A[4] * A[6]);
}

CPFEM_HD void inv3(const double* A, double* Ai) {
  const double c00 = A[4] * A[8] - A[5] * A[7];
  const double c01 = A[5] * A[6] - A[3] * A[8];
  const double c02 = A[3] * A[7] - A[4] * A[6];
  const double det = A[0] * c00 + A[1] * c01 + A[2] * c02;
  const double id = 1.0 / det;
  Ai[0] = c00 * id;
  Ai[1] = (A[2] * A[7] - A[1] * A[8]) * id;
  Ai[2] = (A[1] * A[5] - A[2] * A[4]) * id;
  Ai[3] = c01 * id;
  Ai[4] = (A[0] * A[8] - A[2] * A[6]) * id;
  Ai[5] = (A[2] * A[3] - A[0] * A[5]) * id;
  Ai[6] = c02 * id;
  Ai[7] = (A[1] * A[6] - A[0] * A[7]) * id;
  Ai[8] = (A[0] * A[4] - A[1] * A[3]) * id;
}

// Cubic elastic constants of one Gauss point (the material's, or its phase's row).
struct Cub {
  double C11, C12, C44;
};

// Cubic stiffness applied to a symmetric tensor in 6-component form
// (11,22,33,23,13,12), tensor components (not engineering shears).
CPFEM_HD void cubic_apply(const Cub& m, const double* e, double* t) {
  t[0] = fma(m.C11, e[0], m.C12 * (e[1] + e[2]));
  t[1] = fma(m.C11, e[1], m.C12 * (e[0] + e[2]));
  t[2] = fma(m.C11, e[2], m.C12 * (e[0] + e[1]));
  const double c2 = 2.0 * m.C44;
  t[3] = c2 * e[3];
  t[4] = c2 * e[4];
  t[5] = c2 * e[5];
}

CPFEM_HD void cubic_apply(const Cub& m, const float* e, float* t) {
  const float c11 = (float)m.C11, c12 = (float)m.C12, c2 = (float)(2.0 * m.C44);
  t[0] = fmaf(c11, e[0], c12 * (e[1] + e[2]));
  t[1] = fmaf(c11, e[1], c12 * (e[0] + e[2]));
  t[2] = fmaf(c11, e[2], c12 * (e[0] + e[1]));
  t[3] = c2 * e[3];
  t[4] = c2 * e[4];
  t[5] = c2 * e[5];
}

CPFEM_HD double cp_fma(double a, double b, double c) { return fma(a, b, c); }
CPFEM_HD float cp_fma(float a, float b, float c) { return fmaf(a, b, c); }
CPFEM_HD double cp_abs(double a) { return fabs(a); }
CPFEM_HD float cp_abs(float a) { return fabsf(a); }

// FP64 <-> FP32 by integer operations on the bit patterns.  GB300 issues the conversion
// instructions on its FP64 pipe at the DFMA rate; these run on the integer pipes
// (measured on GB300: 8.5x (FP64 -> FP32) and 4.4x (FP32 -> FP64) the conversion
// instructions' throughput).  f32_of truncates the mantissa to 23 bits (error < 2^-23
// relative), flushes magnitudes below FP32's normal range to a signed zero and saturates
// above it to a signed infinity (a NaN becomes an infinity).  f64_of is exact for normal
// floats and infinities, keeps a NaN a NaN and flushes FP32 subnormals to zero.  Host
// builds use the plain conversions.
CPFEM_HD float f32_of(double v) {
#ifdef __CUDA_ARCH__
  const unsigned hi = (unsigned)__double2hiint(v), lo = (unsigned)__double2loint(v);
  const unsigned sign = hi & 0x80000000u;
  const int e = (int)((hi >> 20) & 0x7FFu) - 1023 + 127;
  const unsigned bits = (e <= 0) ? sign
                        : (e >= 255) ? (sign | 0x7F800000u)
                                     : (sign | ((unsigned)e << 23) | ((hi & 0xFFFFFu) << 3) | (lo >> 29));
  return __uint_as_float(bits);
#else
  return (float)v;
#endif
}
CPFEM_HD double f64_of(float f) {
#ifdef __CUDA_ARCH__
  const unsigned u = __float_as_uint(f);
  const unsigned sign = u & 0x80000000u, ex = (u >> 23) & 0xFFu, mant = u & 0x7FFFFFu;
  const unsigned hi = (ex == 0u) ? sign : (sign | ((ex == 255u ? 2047u : ex + 896u) << 20) | (mant >> 3));
  const unsigned lo = (ex == 0u) ? 0u : (mant << 29);
  return __hiloint2double((int)hi, (int)lo);
#else
  return (double)f;
#endif
}
CPFEM_HD float to_f32(float v) { return v; }
CPFEM_HD float to_f32(double v) { return f32_of(v); }
CPFEM_HD double to_f64(double v) { return v; }
CPFEM_HD double to_f64(float v) { return f64_of(v); }
// a value in the precision T of a computation (FP32 through f32_of)
template <typename T>
CPFEM_HD T to_prec(double v);
template <>
CPFEM_HD double to_prec<double>(double v) { return v; }
template <>
CPFEM_HD float to_prec<float>(double v) { return f32_of(v); }

// In-register LU with partial pivoting of an n x n matrix (FP64, or FP32 for a Newton
// direction that need not be exact); all indices are static so the matrix stays in
// registers.  Row swaps are done with predicated exchanges.
template <int n, typename T>
CPFEM_HD void lu_factor(T* A, int* perm, T* dinv) {
#pragma unroll
  for (int i = 0; i < n; ++i) perm[i] = i;
#pragma unroll
  for (int k = 0; k < n; ++k) {
    int p = k;
    T best = cp_abs(A[k * n + k]);
#pragma unroll
    for (int i = k + 1; i < n; ++i) {
      const T v = cp_abs(A[i * n + k]);
      if (v > best) { best = v; p = i; }
    }
#pragma unroll
    for (int i = k + 1; i < n; ++i) {
      if (p == i) {
#pragma unroll
        for (int j = 0; j < n; ++j) {
          const T t = A[k * n + j];
          A[k * n + j] = A[i * n + j];
          A[i * n + j] = t;
        }
        const int t = perm[k];
        perm[k] = perm[i];
        perm[i] = t;
      }
    }
    const T inv = T(1) / A[k * n + k];
    dinv[k] = inv;
#pragma unroll
    for (int i = k + 1; i < n; ++i) {
      const T l = A[i * n + k] * inv;
      A[i * n + k] = l;
#pragma unroll
      for (int j = k + 1; j < n; ++j) A[i * n + j] = cp_fma(-l, A[k * n + j], A[i * n + j]);
    }
  }
}

// Solve with the factors of lu_factor; b is overwritten by x.
template <int n, typename T>
CPFEM_HD void lu_solve(const T* LU, const int* perm, const T* dinv, T* b) {
  T y[n];
#pragma unroll
  for (int i = 0; i < n; ++i) {
    T v = T(0);
#pragma unroll
    for (int j = 0; j < n; ++j) v = (perm[i] == j) ? b[j] : v;
    y[i] = v;
  }
#pragma unroll
  for (int i = 0; i < n; ++i)
#pragma unroll
    for (int j = 0; j < i; ++j) y[i] = cp_fma(-LU[i * n + j], y[j], y[i]);
#pragma unroll
  for (int i = n - 1; i >= 0; --i) {
#pragma unroll
    for (int j = i + 1; j < n; ++j) y[i] = cp_fma(-LU[i * n + j], y[j], y[i]);
    y[i] = y[i] * dinv[i];
  }
#pragma unroll
  for (int i = 0; i < n; ++i) b[i] = y[i];
}

}  // namespace cpfem
