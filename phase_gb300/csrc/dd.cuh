// Float-float ("double-single") arithmetic for the mixed-precision solver.
//
// A value is the unevaluated sum hi + lo of two FP32 numbers with
// |lo| <= ulp(hi)/2: about 48 significant bits, computed entirely on the
// FP32 pipes (GB300 executes FP64 at a small fraction of its FP32 rate).
// The building blocks are the classical error-free transformations:
//   TwoSum      (Knuth, TAOCP vol. 2): a + b = s + e exactly
//   FastTwoSum  (Dekker 1971):         the same when |a| >= |b|
//   TwoProduct  via FMA:               a * b = p + e exactly
// the accurate double-word addition (two TwoSums, as in Hida, Li & Bailey
// 2001) and the Dot2 compensated accumulation of Ogita, Rump & Oishi 2005
// for sums of products (SpMV rows, dot products, triangular-solve rows).
// The __f*_rn intrinsics keep the compiler from contracting a product into
// a following addition or reassociating, which would break the
// transformations.  Values are stored as float2 {hi, lo} (8 bytes, the
// same traffic as FP64).
#pragma once

#include <cuda_runtime.h>

#include "kernels.cuh"

namespace pg {

__device__ __forceinline__ float2 two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return make_float2(s, e);
}

// requires |a| >= |b| (or a == 0)
__device__ __forceinline__ float2 fast_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return make_float2(s, __fsub_rn(b, __fsub_rn(s, a)));
}

__device__ __forceinline__ float2 dd_add(float2 x, float2 y) {
  float2 s = two_sum(x.x, y.x);
  const float2 t = two_sum(x.y, y.y);
  s = fast_two_sum(s.x, __fadd_rn(s.y, t.x));
  return fast_two_sum(s.x, __fadd_rn(s.y, t.y));
}

__device__ __forceinline__ float2 dd_neg(float2 x) {
  return make_float2(-x.x, -x.y);
}

__device__ __forceinline__ float2 dd_sub(float2 x, float2 y) {
  return dd_add(x, dd_neg(y));
}

__device__ __forceinline__ float2 dd_mul(float2 x, float2 y) {
  const float p = __fmul_rn(x.x, y.x);
  float e = __fmaf_rn(x.x, y.x, -p);
  e = __fmaf_rn(x.x, y.y, e);
  e = __fmaf_rn(x.y, y.x, e);
  return fast_two_sum(p, e);
}

// Compensated accumulator (Dot2): s is the running FP32 sum, c collects the
// rounding errors of the additions and products.  Only the one FP32 add per
// term on s is a serial dependence.
struct DdAcc {
  float s, c;
};

__device__ __forceinline__ DdAcc dd_acc(float2 x) { return DdAcc{x.x, x.y}; }

// a += x * y
__device__ __forceinline__ void dd_acc_fma(DdAcc &a, float2 x, float2 y) {
  const float p = __fmul_rn(x.x, y.x);
  const float pe = __fmaf_rn(x.y, y.x, __fmaf_rn(x.x, y.y, __fmaf_rn(x.x, y.x, -p)));
  const float2 t = two_sum(a.s, p);
  a.s = t.x;
  a.c = __fadd_rn(a.c, __fadd_rn(t.y, pe));
}

// a += w * y for an FP32 w (a factor weight stored in FP32)
__device__ __forceinline__ void dd_acc_fma_f(DdAcc &a, float w, float2 y) {
  const float p = __fmul_rn(w, y.x);
  const float pe = __fmaf_rn(w, y.y, __fmaf_rn(w, y.x, -p));
  const float2 t = two_sum(a.s, p);
  a.s = t.x;
  a.c = __fadd_rn(a.c, __fadd_rn(t.y, pe));
}

// x * d for an FP32 d
__device__ __forceinline__ float2 dd_mul_f(float2 x, float d) {
  const float p = __fmul_rn(x.x, d);
  const float e = __fmaf_rn(x.y, d, __fmaf_rn(x.x, d, -p));
  return fast_two_sum(p, e);
}

// a += x
__device__ __forceinline__ void dd_acc_add(DdAcc &a, float2 x) {
  const float2 t = two_sum(a.s, x.x);
  a.s = t.x;
  a.c = __fadd_rn(a.c, __fadd_rn(t.y, x.y));
}

// merges two accumulators (tree reductions)
__device__ __forceinline__ void dd_acc_merge(DdAcc &a, const DdAcc &b) {
  const float2 t = two_sum(a.s, b.s);
  a.s = t.x;
  a.c = __fadd_rn(__fadd_rn(a.c, b.c), t.y);
}

__device__ __forceinline__ float2 dd_value(const DdAcc &a) {
  return two_sum(a.s, a.c);
}

// conversions (these use the FP64 pipe: keep them off the per-iteration path)
__device__ __forceinline__ float2 dd_from(double v) {
  const float hi = __double2float_rn(v);
  return make_float2(hi, __double2float_rn(v - (double)hi));
}

__device__ __forceinline__ double dd_to_double(float2 x) {
  return (double)x.x + (double)x.y;
}

__device__ __forceinline__ double dd_acc_to_double(const DdAcc &a) {
  return (double)a.s + (double)a.c;
}

// Input of a float-float preconditioner application with the fused
// BiCGStab update (modes as pre_input in kernels.cuh):
//   mode 1: p = r + beta (p - omega v), written back to pv
//   mode 2: s = r - alpha v,            written to pv
__device__ __forceinline__ float2 dd_pre_combine(int mode, float2 ri,
                                                 float2 pi, float2 vi,
                                                 const KScalars *sc) {
  if (mode == 1)
    return dd_add(ri, dd_mul(sc->beta_dd, dd_sub(pi, dd_mul(sc->omega_dd, vi))));
  if (mode == 2) return dd_sub(ri, dd_mul(sc->alpha_dd, vi));
  return pi;
}

__device__ __forceinline__ float2 dd_pre_input(int mode, int i,
                                               const float2 *r, float2 *pv,
                                               const float2 *v,
                                               const KScalars *sc) {
  const float2 zero = make_float2(0.f, 0.f);
  const float2 val = dd_pre_combine(mode, mode ? r[i] : zero,
                                    mode != 2 ? pv[i] : zero,
                                    mode ? v[i] : zero, sc);
  if (mode) pv[i] = val;
  return val;
}

}  // namespace pg
