// Anchored TaylorF2 phase recurrence shared by the bin-walking kernels: the
// Taylor coefficients of the phase about an anchor bin from the per-analysis
// tables of the basis functions, their forward differences in 0.64 fixed
// point, and the choice of anchor interval and polynomial degree.
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

// Forward differences D[0..6] (0.64 fixed point, cycles) of the phase
// polynomial about anchor bin k, truncated at degree deg: the float-float
// dot products A_n = sum_b c_b T_n,b(k) (orders 0..3 float-float, 4..6
// float32) and Delta_m = m! sum_n S(n, m) A_n (Stirling numbers).  ch / cl:
// the point's basis coefficients (index kNumBasis: the constant).
__device__ __forceinline__ void anchor_differences(const float* anchors, int64_t k, const float* ch, const float* cl,
                                                   int deg, uint64_t* D) {
  const float* an = anchors + (k / kAnchorStep) * kAnchorFloats;
  float Ah[kAnchorFF], Al[kAnchorFF], Af[kAnchorOrders - kAnchorFF];
#pragma unroll
  for (int n = 0; n < kAnchorFF; ++n) {
    float sh = n == 0 ? ch[kNumBasis] : 0.f, sl = n == 0 ? cl[kNumBasis] : 0.f;
#pragma unroll
    for (int b = 0; b < kNumBasis; ++b)
      ff_mac(sh, sl, ch[b], cl[b], __ldg(an + n * kNumBasis + b),
             __ldg(an + kAnchorOrders * kNumBasis + n * kNumBasis + b));
    Ah[n] = sh;
    Al[n] = sl;
  }
#pragma unroll
  for (int n = kAnchorFF; n < kAnchorOrders; ++n) {
    float sf = 0.f;
#pragma unroll
    for (int b = 0; b < kNumBasis; ++b) sf = __fmaf_rn(ch[b], __ldg(an + n * kNumBasis + b), sf);
    Af[n - kAnchorFF] = sf;
  }
  const float A4 = Af[0], A5 = deg >= 5 ? Af[1] : 0.f, A6 = deg >= 6 ? Af[2] : 0.f;
  float d1h = Ah[1], d1l = Al[1];
  ff_add(d1h, d1l, Ah[2], Al[2]);
  ff_add(d1h, d1l, Ah[3], Al[3]);
  ff_add(d1h, d1l, __fadd_rn(__fadd_rn(A4, A5), A6), 0.f);
  float d2h = Ah[2], d2l = Al[2];
  ff_scale(d2h, d2l, 2.f);
  float t3h = Ah[3], t3l = Al[3];
  ff_scale(t3h, t3l, 6.f);
  ff_add(d2h, d2l, t3h, t3l);
  ff_add(d2h, d2l, lin3(14.f, A4, 30.f, A5, 62.f, A6), 0.f);
  float d3h = Ah[3], d3l = Al[3];
  ff_scale(d3h, d3l, 6.f);
  ff_add(d3h, d3l, lin3(36.f, A4, 150.f, A5, 540.f, A6), 0.f);
  D[0] = to_fixed(Ah[0], Al[0]);
  D[1] = to_fixed(d1h, d1l);
  D[2] = to_fixed(d2h, d2l);
  D[3] = to_fixed(d3h, d3l);
  D[4] = to_fixed(lin3(24.f, A4, 240.f, A5, 1560.f, A6), 0.f);
  D[5] = to_fixed(__fmaf_rn(1800.f, A6, __fmul_rn(120.f, A5)), 0.f);
  D[6] = to_fixed(__fmul_rn(720.f, A6), 0.f);
}

}  // namespace gwl
