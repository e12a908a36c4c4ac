// sfd_common.cuh -- shared device types and arithmetic for the GB300 boundary-
// integral engine: FP64 complex helpers and double-float ("df", an unevaluated
// pair of FP32 numbers hi + lo carrying ~48 significant bits) arithmetic.
//
// Double-float building blocks follow the classical error-free transforms
// (Knuth two-sum, Dekker/FMA two-product; Hida-Li-Bailey "double-double"
// arithmetic restated for float pairs).  They let the O(N^2) kernel sums run on
// the FP32 pipes (~70 TFLOP/s on GB300) instead of the FP64 pipes (~1.2 TFLOP/s)
// while keeping ~1e-13 relative accuracy.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#define SFD_PI 3.14159265358979323846

// ---------------------------------------------------------------- FP64 complex
struct cd {
  double re, im;
};
__host__ __device__ __forceinline__ cd mk(double r, double i) { return cd{r, i}; }
__host__ __device__ __forceinline__ cd operator+(cd a, cd b) { return {a.re + b.re, a.im + b.im}; }
__host__ __device__ __forceinline__ cd operator-(cd a, cd b) { return {a.re - b.re, a.im - b.im}; }
__host__ __device__ __forceinline__ cd operator*(cd a, cd b) {
  return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}
__host__ __device__ __forceinline__ cd operator*(double s, cd a) { return {s * a.re, s * a.im}; }
__host__ __device__ __forceinline__ cd cconj(cd a) { return {a.re, -a.im}; }
__host__ __device__ __forceinline__ cd cmul_i(cd a) { return {-a.im, a.re}; }  // i * a
__host__ __device__ __forceinline__ double cabs2(cd a) { return a.re * a.re + a.im * a.im; }
// a / b by the textbook formula conj(b) / |b|^2 (operands here are O(1) and far
// from overflow, so no Smith scaling is needed).
__host__ __device__ __forceinline__ cd cdiv(cd a, cd b) {
  double d = 1.0 / (b.re * b.re + b.im * b.im);
  return {(a.re * b.re + a.im * b.im) * d, (a.im * b.re - a.re * b.im) * d};
}

// ---------------------------------------------------------------- double-float
struct df {
  float hi, lo;
};

// s + e = a + b exactly (Knuth).
__device__ __forceinline__ df two_sum(float a, float b) {
  float s = __fadd_rn(a, b);
  float bb = __fsub_rn(s, a);
  float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return {s, e};
}
// requires |a| >= |b|
__device__ __forceinline__ df quick_two_sum(float a, float b) {
  float s = __fadd_rn(a, b);
  float e = __fsub_rn(b, __fsub_rn(s, a));
  return {s, e};
}
// p + e = a * b exactly (FMA).
__device__ __forceinline__ df two_prod(float a, float b) {
  float p = __fmul_rn(a, b);
  float e = __fmaf_rn(a, b, -p);
  return {p, e};
}
__device__ __forceinline__ df df_from_double(double x) {
  float hi = __double2float_rn(x);
  float lo = __double2float_rn(x - (double)hi);
  return {hi, lo};
}
__host__ __device__ __forceinline__ double df_to_double(df a) { return (double)a.hi + (double)a.lo; }

// a + b ("sloppy" variant: exact hi two-sum, lo parts added in FP32).  When
// a.hi and b.hi nearly cancel the two-sum is exact and the result keeps the
// lo-part difference to FP32 relative accuracy.
__device__ __forceinline__ df df_add(df a, df b) {
  df s = two_sum(a.hi, b.hi);
  float e = __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo));
  return quick_two_sum(s.hi, e);
}
__device__ __forceinline__ df df_neg(df a) { return {-a.hi, -a.lo}; }
__device__ __forceinline__ df df_sub(df a, df b) { return df_add(a, df_neg(b)); }
__device__ __forceinline__ df df_mul(df a, df b) {
  df p = two_prod(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, p.lo));
  return quick_two_sum(p.hi, e);
}
// 1 / a: hardware reciprocal estimate refined by one Newton step evaluated in
// double-float (r = r0 + r0 (1 - a r0)).
__device__ __forceinline__ df df_rcp(df a) {
  float r0;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r0) : "f"(a.hi));
  df p = two_prod(a.hi, r0);                      // a.hi * r0 = p.hi + p.lo
  float e = __fsub_rn(__fsub_rn(1.0f, p.hi), p.lo);  // 1 - p.hi is exact near 1
  e = __fmaf_rn(-a.lo, r0, e);                    // - a.lo * r0
  return quick_two_sum(r0, __fmul_rn(r0, e));
}

// a - b: hi parts differenced exactly (two-sum), lo parts in FP32, then
// renormalised.  When a and b are close the exact hi difference is small and
// the lo difference is not, so the renormalisation is required: df_mul and
// df_sqsum drop lo * lo products, which is only safe for |lo| <= ulp(hi).
__device__ __forceinline__ df df_diff(df a, df b) {
  df s = two_sum(a.hi, -b.hi);
  float lo = __fadd_rn(s.lo, __fsub_rn(a.lo, b.lo));
  return two_sum(s.hi, lo);
}
// x^2 + y^2 for double-float x, y (normalised result).
__device__ __forceinline__ df df_sqsum(df x, df y) {
  df px = two_prod(x.hi, x.hi);
  float ex = __fmaf_rn(2.0f * x.hi, x.lo, px.lo);
  df py = two_prod(y.hi, y.hi);
  float ey = __fmaf_rn(2.0f * y.hi, y.lo, py.lo);
  df s = two_sum(px.hi, py.hi);
  return quick_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(ex, ey)));
}
// FP32 reciprocal estimate (about 1 ulp), for the FP32 correction passes.
__device__ __forceinline__ float rcp_approx(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// Double-float complex.
struct dfc {
  df re, im;
};

// ---------------------------------------------------------------- status word
// Per-surface status bits written by kernels and read by the host once per call.
enum : uint32_t {
  SFD_ST_OK = 0u,
  SFD_ST_NONFINITE = 1u << 0,        // NaN / Inf met in the state or a result
  SFD_ST_PIVOT_SWAP = 1u << 1,       // |l_ij| > 1: partial pivoting would have swapped rows
  SFD_ST_ZERO_PIVOT = 1u << 2,       // a pivot was zero / below the breakdown threshold
  SFD_ST_REFINE_STALL = 1u << 3,     // iterative refinement did not reach its tolerance
  SFD_ST_REFACTORED = 1u << 4,       // informational: the preconditioner was rebuilt
  SFD_ST_TIMEOUT = 1u << 5,          // a bounded wait in a kernel ran out (kernel skipped its work)
};

#define SFD_CUDA_OK(expr)                       \
  do {                                          \
    cudaError_t _e = (expr);                    \
    if (_e != cudaSuccess) return sfd_fail(_e); \
  } while (0)
