// Anchored TaylorF2 phase shared by the bin-walking kernels: the Taylor
// coefficients of the phase about an anchor bin from the per-analysis tables
// of the basis functions, the choice of anchor interval and polynomial
// degree, and packed float-pair arithmetic.
#pragma once

#include <cstdint>

#include "gwl_device.cuh"
#include "gwl_internal.h"

namespace gwl {

// ff helpers for the anchor set-up (all float32 operations, error-free transforms)
__device__ __forceinline__ void ff_add(float& hi, float& lo, float bh, float bl) {
  const float s = __fadd_rn(hi, bh);
  const float bb = __fsub_rn(s, hi);
  float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(bh, bb));
  e = __fadd_rn(e, __fadd_rn(lo, bl));
  hi = __fadd_rn(s, e);
  lo = __fsub_rn(e, __fsub_rn(hi, s));
}

__device__ __forceinline__ void ff_scale(float& hi, float& lo, float k) {
  const float p = __fmul_rn(hi, k);
  const float e = __fmaf_rn(hi, k, -p);
  hi = p;
  lo = __fmaf_rn(lo, k, e);
}

// hi + lo += x with TwoSum (Knuth): the float-float accumulation of the
// 8-bin float32 partial sums
__device__ __forceinline__ void two_sum_acc(float& hi, float& lo, float x) {
  const float s = __fadd_rn(hi, x);
  const float bb = __fsub_rn(s, hi);
  const float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(x, bb));
  hi = s;
  lo = __fadd_rn(lo, e);
}

// a0 x0 + a1 x1 + a2 x2 with a fixed operation order (no compiler contraction)
__device__ __forceinline__ float lin3(float a0, float x0, float a1, float x1, float a2, float x2) {
  return __fmaf_rn(a2, x2, __fmaf_rn(a1, x1, __fmul_rn(a0, x0)));
}

// (hi + lo) modulo one cycle as 0.64 fixed point
__device__ __forceinline__ uint64_t to_fixed(float hi, float lo) {
  float r = __fsub_rn(hi, rintf(hi));
  if (r >= 0.5f) r -= 1.0f;
  float q = __fsub_rn(lo, rintf(lo));
  if (q >= 0.5f) q -= 1.0f;
  const long long a = __float2ll_rn(r * 18446744073709551616.0f);
  const long long b = __float2ll_rn(q * 18446744073709551616.0f);
  return (uint64_t)(a + b);
}

// Largest anchor interval J (power of two, 8..256 bins) for which, at a chunk
// starting at bin k0 with Newtonian phase magnitude N cycles there, the
// degree-6 Taylor remainder stays below 1e-9 cycle and the float32 orders
// 4..6 below 1e-2 * 6e-8 cycle (factor 8 of margin for the PN terms).
// 256 keeps the fixed-point quantisation C(J,6) 2^-65 below 1e-8 cycle.
// Returns 0 when even J = 8 violates the bound (low bins of short segments,
// where f changes by a large fraction per bin): the chunk then evaluates the
// phase at every bin in float-float from the per-bin basis table.
__device__ __forceinline__ int anchor_interval(float n_cycles, float k0) {
  for (int J = 256; J >= 8; J >>= 1) {
    const float x = (float)J / k0;
    const float x2 = x * x, x4 = x2 * x2, x7 = x4 * x2 * x;
    if (n_cycles * x7 <= 3.1e-11f && n_cycles * x4 <= 4.5e-4f) return J;
  }
  return 0;
}

// Degree of the phase polynomial about an anchor: the lowest of 4, 5, 6 whose
// Taylor remainder N x^(deg + 1) stays within the bound of anchor_interval
// (N the Newtonian phase in cycles at the anchor, x = J / k).
__device__ __forceinline__ int anchor_degree(float n_cycles, float x) {
  const float x5 = x * x * x * x * x;
  if (n_cycles * x5 <= 3.1e-11f) return 4;
  if (n_cycles * x5 * x <= 3.1e-11f) return 5;
  return 6;
}

// Taylor coefficients A_n of the phase polynomial about anchor bin k, in
// cycles: Phi(k + j) = sum_n A_n j^n.  A_n = sum_b c_b T_n,b(k) from the
// per-analysis Taylor tables of the basis functions, orders 0..3 as
// float-float dot products and 4..6 in float32.  ch / cl: the point's basis
// coefficients (index kNumBasis: the constant).
struct AnchorTaylor {
  float h[kAnchorFF], l[kAnchorFF];   // orders 0..3, float-float
  float f[kAnchorOrders - kAnchorFF]; // orders 4..6
};

__device__ __forceinline__ void anchor_taylor(const float* anchors, int64_t k, const float* ch, const float* cl,
                                              AnchorTaylor& t) {
  const float* an = anchors + (k / kAnchorStep) * kAnchorFloats;
#pragma unroll
  for (int n = 0; n < kAnchorFF; ++n) {
    float sh = n == 0 ? ch[kNumBasis] : 0.f, sl = n == 0 ? cl[kNumBasis] : 0.f;
#pragma unroll
    for (int b = 0; b < kNumBasis; ++b)
      ff_mac(sh, sl, ch[b], cl[b], __ldg(an + n * kNumBasis + b),
             __ldg(an + kAnchorOrders * kNumBasis + n * kNumBasis + b));
    t.h[n] = sh;
    t.l[n] = sl;
  }
#pragma unroll
  for (int n = kAnchorFF; n < kAnchorOrders; ++n) {
    float sf = 0.f;
#pragma unroll
    for (int b = 0; b < kNumBasis; ++b) sf = __fmaf_rn(ch[b], __ldg(an + n * kNumBasis + b), sf);
    t.f[n - kAnchorFF] = sf;
  }
}

// ---------------------------------------------------------------------------
// Packed float pairs: the sm_100-family f32x2 instructions do two IEEE
// round-to-nearest float32 operations in one issue slot.  Lane x and lane y
// are independent; the pair lives in one 64-bit register pair.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) {
  float2 r;
  asm("{\n\t.reg .b64 ra, rb, rc, rd;\n\t"
      "mov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\tmov.b64 rc, {%6, %7};\n\t"
      "fma.rn.f32x2 rd, ra, rb, rc;\n\tmov.b64 {%0, %1}, rd;\n\t}"
      : "=f"(r.x), "=f"(r.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y), "f"(c.x), "f"(c.y));
  return r;
}

__device__ __forceinline__ float2 mul2(float2 a, float2 b) {
  float2 r;
  asm("{\n\t.reg .b64 ra, rb, rd;\n\t"
      "mov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t"
      "mul.rn.f32x2 rd, ra, rb;\n\tmov.b64 {%0, %1}, rd;\n\t}"
      : "=f"(r.x), "=f"(r.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
  return r;
}

__device__ __forceinline__ float2 add2(float2 a, float2 b) {
  float2 r;
  asm("{\n\t.reg .b64 ra, rb, rd;\n\t"
      "mov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t"
      "add.rn.f32x2 rd, ra, rb;\n\tmov.b64 {%0, %1}, rd;\n\t}"
      : "=f"(r.x), "=f"(r.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
  return r;
}

}  // namespace gwl
