// df.cuh — double-float arithmetic on the FP32 pipe. A value is carried as
// hi + lo (two floats), about 48 significant bits. Products and sums use the
// error-free transformations of double-double arithmetic (TwoProd by FMA;
// TwoSum, Knuth 1969 and Dekker 1971; as in Hida, Li & Bailey 2001). GB300's
// FP32 pipe issues about 70 times the FMAs of its FP64 pipe, which pays where
// the products outnumber the operands' conversions (the batched solver's
// block products). The __f*_rn intrinsics are never contracted into FMAs,
// which would break the transformations.
#pragma once

#include <cstdint>

namespace sed {

// v = h + l with h = v rounded to 24 bits and l the remainder rounded to 24
// bits (conversion instructions).
__device__ __forceinline__ void df_split(double v, float& h, float& l) {
  h = __double2float_rn(v);
  l = __double2float_rn(v - (double)h);
}

// (S, E) += (ah + al)(bh + bl): S collects the rounded products exactly (the
// TwoSum error goes to E), E the product errors and the cross terms; al*bl
// (below 2^-48 of the product) is dropped.
__device__ __forceinline__ void df_mac(float ah, float al, float bh, float bl, float& S, float& E) {
  float const p = __fmul_rn(ah, bh);
  float e = __fmaf_rn(ah, bh, -p);
  e = __fmaf_rn(ah, bl, e);
  e = __fmaf_rn(al, bh, e);
  float const s = __fadd_rn(S, p);
  float const bb = __fsub_rn(s, S);
  float const err = __fadd_rn(__fsub_rn(S, __fsub_rn(s, bb)), __fsub_rn(p, bb));
  S = s;
  E = __fadd_rn(E, __fadd_rn(err, e));
}

// (h, l) -= (S + E), renormalised so that |l| <= ulp(h) / 2.
__device__ __forceinline__ void df_sub(float& h, float& l, float S, float E) {
  float const s = __fsub_rn(h, S);
  float const bb = __fsub_rn(s, h);
  float const err = __fadd_rn(__fsub_rn(h, __fsub_rn(s, bb)), __fsub_rn(-S, bb));
  float const t = __fadd_rn(err, __fsub_rn(l, E));
  h = __fadd_rn(s, t);  // TwoSum(s, t): t may exceed s after cancellation
  float const b2 = __fsub_rn(h, s);
  l = __fadd_rn(__fsub_rn(s, __fsub_rn(h, b2)), __fsub_rn(t, b2));
}

// (h, l) = (ah + al)(bh + bl), renormalised (al bl dropped).
__device__ __forceinline__ void df_mul(float ah, float al, float bh, float bl, float& h, float& l) {
  float const p = __fmul_rn(ah, bh);
  float e = __fmaf_rn(ah, bh, -p);
  e = __fmaf_rn(ah, bl, e);
  e = __fmaf_rn(al, bh, e);
  h = __fadd_rn(p, e);
  l = __fsub_rn(e, __fsub_rn(h, p));
}

}  // namespace sed
