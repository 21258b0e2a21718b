// Multi-banding with the IFFT-FFT <h|h> (bilby/gw/likelihood/multiband.py:
// 613-650, 760-779; Morisaki, arXiv:2104.07813, section 3.3).
//
// For a band b >= 1 of M = Mbs[b] samples and each detector the reference
// forms W_m = sqrt(w_k) s_k at m = K_s + (k - k_b) (zero at the other m <= M/2;
// s_k the detector response at banded frequency k), y = irfft(W) (M real
// samples), hbc = M zeros followed by y (2M samples), X = rfft(hbc) (M + 1
// bins) and (4 / That_b) sum_k |X_k|^2 Re I_k.  Since
//   X_k = (-1)^k sum_n y_n exp(-i pi k n / M),
// the even bins are X_2j = (DFT_M y)_j = W_j: their terms are a fixed weight
// times |s_k|^2, which the caller folds into the quadratic coefficients.  The
// odd bins are |X_2j+1| = |Z_j| with Z_j = sum_n y_n exp(-i pi n (2j + 1) / M),
// the DFT of y_n exp(-i pi n / M); this file computes their part.
//
// One CTA per (point, pair of detectors) and band, the two detectors' real
// transforms packed in one complex one:
//   C = W_d1 + i W_d2 over the Hermitian extensions (C_(M-m) = conj W_d1,m
//       + i conj W_d2,m), so that IDFT(C) / M = y_d1 + i y_d2;
//   the inverse DFT by decimation in frequency (natural order in,
//   bit-reversed out), times exp(-i pi n / M) / M at the bit-reversed
//   positions, the forward DFT by decimation in time (bit-reversed in,
//   natural out): F = Z_d1 + i Z_d2;
//   Z_d1,j = (F_j + conj F_(M-1-j)) / 2, Z_d2,j = (F_j - conj F_(M-1-j)) / 2i
//   (a real y has Z_(M-1-j) = conj Z_j), for j < M / 2.
// float64 throughout, in place, radix-4 passes (one radix-2 stage more for
// an odd log2 M).  The transform lives in
// shared memory up to 2^kMbFftSmemLog2 samples, above that in a global slot per
// CTA (a persistent grid of one CTA per SM, whose slots stay in L2).  The
// partner detector of a point is fixed (d, d + 1), so a point's result does
// not depend on the batch it is evaluated in.
//
// Mixed precision (TaylorF2): k_mb_hh_fft32 forms the banded values as the
// mixed multi-banding kernel does (float-float phase basis reduced to 0.64
// fixed point, the time shift exact per band, sincospi in float32, the
// amplitude from a float table of sqrt(w) f^(-7/6)), runs the same passes in
// float32 and sums in float64.  Its error bound per (band, detector, point)
// is kFft32Err u sqrt(log2 M + 2) sqrt(sum |Z|^2 o^2) sqrt(sum |Z|^2)
// (independent rounding of the banded values and of the two transforms;
// Cauchy-Schwarz on the weighted sum); a point whose bound, summed over bands
// and detectors, exceeds the tolerance is listed and recomputed by the
// float64 kernel.  The bound is on <h|h>/2, the lnL's change without the
// distance table; with it the float64 transforms run instead.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>

#include "gwl_device.cuh"
#include "gwl_internal.h"
#include "gwl_marg_common.cuh"
#include "gwl_math.cuh"
#include "gwl_phase.cuh"

namespace gwl {

namespace {

constexpr int kMbFftThreads = 512;
// float32 transforms live in shared memory up to 2^kMbFft32SmemLog2 samples;
// a longer one runs in a global slot with blocks of 2^kMbFft32BlockLog2
// samples in shared memory (64 KB: two CTAs per SM, as the register cap of
// the float32 kernel allows)
constexpr int kMbFft32SmemLog2 = 14;
constexpr int kMbFft32BlockLog2 = 13;
// error-bound coefficient of the float32 path, times u sqrt(log2 M + 2): the
// rounding of the banded values and of the passes is independent from value
// to value, so the transform's error grows as the square root of its depth.
// Measured on tf2_128s (1024 prior draws and 1024 templates at 0.05-120 Mpc,
// <h|h> up to 4e9) |d<h|h>| <= 1.6e-7 <h|h>, i.e. |d lnL| <= 0.8e-7 <h|h>;
// the bound on |d lnL| is at least 0.5 kFft32Err u sqrt(log2 M + 2) <h|h>
// >= 2.9e-7 <h|h> for M >= 4096 (Cauchy-Schwarz makes the norm product at
// least the sum), a margin of 3.6 or more.
constexpr double kFft32Err = 2.5;
constexpr double kU32 = 5.9604644775390625e-08;  // 2^-24

template <class T>
struct V2;
template <>
struct V2<float> {
  using t = float2;
  static __device__ __forceinline__ float2 make(float x, float y) { return make_float2(x, y); }
};
template <>
struct V2<double> {
  using t = double2;
  static __device__ __forceinline__ double2 make(double x, double y) { return make_double2(x, y); }
};

// The radix-4 twiddles t^1, t^2, t^3 at table index k (t = tw[k]): read
// from the table in float64 (its pipe is the bound there), from one read
// and two complex products in float32 (a read of the table costs more than
// the products; the products add about 2u to the twiddles' rounding).
template <class T>
__device__ __forceinline__ void twiddles3(const typename V2<T>::t* tw, size_t k, typename V2<T>::t& t1,
                                          typename V2<T>::t& t2, typename V2<T>::t& t3) {
  if constexpr (sizeof(T) == sizeof(double)) {
    t1 = __ldg(tw + k);
    t2 = __ldg(tw + 2 * k);
    t3 = __ldg(tw + 3 * k);
  } else {
    t1 = __ldg(tw + k);
    t2 = V2<T>::make(t1.x * t1.x - t1.y * t1.y, 2.f * t1.x * t1.y);
    t3 = V2<T>::make(t2.x * t1.x - t2.y * t1.y, t2.x * t1.y + t2.y * t1.x);
  }
}

// Decimation-in-frequency stages lh_hi down to lh_lo (half-size h = 2^lh) of
// an in-place inverse DFT (unnormalised, sign +) over n = 2^log2n values:
// natural order in, bit-reversed out once every stage down to 0 has run.
// Radix-4 passes, each two radix-2 stages (half-sizes h and q = h / 2) on
// {x0, x1, x2, x3} at i0 + {0, q, 2q, 3q} with W = exp(i pi j / h):
//   z0 = (x0 + x2) + (x1 + x3)        z1 = W^2 ((x0 + x2) - (x1 + x3))
//   z2 = W ((x0 - x2) + i (x1 - x3))  z3 = W^3 ((x0 - x2) - i (x1 - x3))
// then, for an odd number of stages, the radix-2 stage lh_lo.  The stages
// below a block size act inside aligned blocks of that size, so they can run
// on a block alone.  tw[k] = exp(-i pi k / 2^sh), k < 2^(sh + 1).  Each pass
// ends with a barrier.
template <class T>
__device__ __forceinline__ void dif_stages(typename V2<T>::t* buf, int log2n, int lh_hi, int lh_lo,
                                           const typename V2<T>::t* tw, int sh) {
  using C = V2<T>;
  const uint32_t n = 1u << log2n;
  int lh = lh_hi;
  for (; lh >= lh_lo + 1; lh -= 2) {
    const int lq = lh - 1;
    const uint32_t q = 1u << lq;
    for (uint32_t t = threadIdx.x; t < (n >> 2); t += blockDim.x) {
      const uint32_t j = t & (q - 1), i0 = ((t >> lq) << (lq + 2)) + j;
      const auto x0 = buf[i0], x1 = buf[i0 + q], x2 = buf[i0 + 2 * q], x3 = buf[i0 + 3 * q];
      const int s = sh - lh;
      typename V2<T>::t w1, w2, w3;
      twiddles3<T>(tw, (size_t)j << s, w1, w2, w3);
      const T ar = x0.x + x2.x, ai = x0.y + x2.y, br = x1.x + x3.x, bi = x1.y + x3.y;
      const T cr = x0.x - x2.x, ci = x0.y - x2.y, dr = x1.x - x3.x, di = x1.y - x3.y;
      buf[i0] = C::make(ar + br, ai + bi);
      const T er = ar - br, ei = ai - bi;  // times conj(w2)
      buf[i0 + q] = C::make(er * w2.x + ei * w2.y, ei * w2.x - er * w2.y);
      const T fr = cr - di, fi = ci + dr;  // (x0 - x2) + i (x1 - x3), times conj(w1)
      buf[i0 + 2 * q] = C::make(fr * w1.x + fi * w1.y, fi * w1.x - fr * w1.y);
      const T gr = cr + di, gi = ci - dr;  // (x0 - x2) - i (x1 - x3), times conj(w3)
      buf[i0 + 3 * q] = C::make(gr * w3.x + gi * w3.y, gi * w3.x - gr * w3.y);
    }
    __syncthreads();
  }
  if (lh == lh_lo) {  // one radix-2 stage left: (x0 + x1, (x0 - x1) conj(W))
    for (uint32_t t = threadIdx.x; t < (n >> 1); t += blockDim.x) {
      const uint32_t j = t & ((1u << lh) - 1), i0 = ((t >> lh) << (lh + 1)) + j, i1 = i0 + (1u << lh);
      const auto x0 = buf[i0], x1 = buf[i1];
      const auto w = __ldg(tw + ((size_t)j << (sh - lh)));
      const T dx = x0.x - x1.x, dy = x0.y - x1.y;
      buf[i0] = C::make(x0.x + x1.x, x0.y + x1.y);
      buf[i1] = C::make(dx * w.x + dy * w.y, dy * w.x - dx * w.y);
    }
    __syncthreads();
  }
}

// times exp(-i pi p / M) / M at the bit-reversed position of p, for the n =
// 2^log2n values at positions base .. base + n - 1 of a transform of M =
// 2^log2m values.  Ends with a barrier.
template <class T>
__device__ __forceinline__ void modulate(typename V2<T>::t* buf, int log2n, uint32_t base, int log2m,
                                         const typename V2<T>::t* tw, int sh) {
  using C = V2<T>;
  const uint32_t n = 1u << log2n;
  const T inv_m = (T)ldexp(1.0, -log2m);
  for (uint32_t q = threadIdx.x; q < n; q += blockDim.x) {
    const uint32_t p = __brev(base + q) >> (32 - log2m);
    const auto w = __ldg(tw + ((size_t)p << (sh - log2m)));
    const auto x = buf[q];
    buf[q] = C::make((x.x * w.x - x.y * w.y) * inv_m, (x.x * w.y + x.y * w.x) * inv_m);
  }
  __syncthreads();
}

// Decimation-in-time stages lh_lo up to lh_hi (half-size h = 2^lh) of an
// in-place forward DFT (sign -) over n = 2^log2n values: bit-reversed in,
// natural out once every stage from 0 has run.  For an odd number of stages
// the radix-2 stage lh_lo first, then radix-4 passes, each two radix-2
// stages (h and 2h) on {x0, x1, x2, x3} at i0 + {0, h, 2h, 3h} with U =
// exp(-i pi j / 2h), a = x0, b = U^2 x1, c = U x2, d = U^3 x3:
//   z0 = (a + b) + (c + d)    z2 = (a + b) - (c + d)
//   z1 = (a - b) - i (c - d)  z3 = (a - b) + i (c - d)
// Each pass ends with a barrier.
template <class T>
__device__ __forceinline__ void dit_stages(typename V2<T>::t* buf, int log2n, int lh_lo, int lh_hi,
                                           const typename V2<T>::t* tw, int sh) {
  using C = V2<T>;
  const uint32_t n = 1u << log2n;
  int lh = lh_lo;
  if ((lh_hi - lh_lo + 1) & 1) {  // x0 + x1 U, x0 - x1 U
    for (uint32_t t = threadIdx.x; t < (n >> 1); t += blockDim.x) {
      const uint32_t j = t & ((1u << lh) - 1), i0 = ((t >> lh) << (lh + 1)) + j, i1 = i0 + (1u << lh);
      const auto x0 = buf[i0], x1 = buf[i1];
      const auto u = __ldg(tw + ((size_t)j << (sh - lh)));
      const T vx = x1.x * u.x - x1.y * u.y, vy = x1.x * u.y + x1.y * u.x;
      buf[i0] = C::make(x0.x + vx, x0.y + vy);
      buf[i1] = C::make(x0.x - vx, x0.y - vy);
    }
    __syncthreads();
    ++lh;
  }
  for (; lh + 1 <= lh_hi; lh += 2) {
    const uint32_t h = 1u << lh;
    for (uint32_t t = threadIdx.x; t < (n >> 2); t += blockDim.x) {
      const uint32_t j = t & (h - 1), i0 = ((t >> lh) << (lh + 2)) + j;
      const auto x0 = buf[i0], x1 = buf[i0 + h], x2 = buf[i0 + 2 * h], x3 = buf[i0 + 3 * h];
      const int s = sh - lh - 1;
      typename V2<T>::t u1, u2, u3;
      twiddles3<T>(tw, (size_t)j << s, u1, u2, u3);
      const T br = x1.x * u2.x - x1.y * u2.y, bi = x1.x * u2.y + x1.y * u2.x;
      const T cr = x2.x * u1.x - x2.y * u1.y, ci = x2.x * u1.y + x2.y * u1.x;
      const T dr = x3.x * u3.x - x3.y * u3.y, di = x3.x * u3.y + x3.y * u3.x;
      const T pr = x0.x + br, pi = x0.y + bi, mr = x0.x - br, mi = x0.y - bi;
      const T sr = cr + dr, si = ci + di, tr = cr - dr, ti = ci - di;
      buf[i0] = C::make(pr + sr, pi + si);
      buf[i0 + 2 * h] = C::make(pr - sr, pi - si);
      buf[i0 + h] = C::make(mr + ti, mi - tr);      // (a - b) - i (c - d)
      buf[i0 + 3 * h] = C::make(mr - ti, mi + tr);  // (a - b) + i (c - d)
    }
    __syncthreads();
  }
}

// The whole packed transform of M = 2^log2m values in buf: inverse DFT,
// exp(-i pi p / M) / M, forward DFT.  With a block buffer sbuf of 2^log2s <
// M values (shared memory; buf then global), the stages above the block size
// run on buf and the rest block by block in sbuf.
template <class T>
__device__ __forceinline__ void packed_transform(typename V2<T>::t* buf, int log2m, typename V2<T>::t* sbuf,
                                                 int log2s, const typename V2<T>::t* tw, int sh) {
  if (!sbuf || log2s >= log2m) {
    dif_stages<T>(buf, log2m, log2m - 1, 0, tw, sh);
    modulate<T>(buf, log2m, 0, log2m, tw, sh);
    dit_stages<T>(buf, log2m, 0, log2m - 1, tw, sh);
    return;
  }
  dif_stages<T>(buf, log2m, log2m - 1, log2s, tw, sh);
  const uint32_t S = 1u << log2s;
  for (uint32_t b0 = 0; b0 < (1u << log2m); b0 += S) {
    for (uint32_t q = threadIdx.x; q < S; q += blockDim.x) sbuf[q] = buf[b0 + q];
    __syncthreads();
    dif_stages<T>(sbuf, log2s, log2s - 1, 0, tw, sh);
    modulate<T>(sbuf, log2s, b0, log2m, tw, sh);
    dit_stages<T>(sbuf, log2s, 0, log2s - 1, tw, sh);
    for (uint32_t q = threadIdx.x; q < S; q += blockDim.x) buf[b0 + q] = sbuf[q];
    __syncthreads();
  }
  dit_stages<T>(buf, log2m, log2s, log2m - 1, tw, sh);
}

// hi + lo += z (w_hi + w_lo): the product's rounding error by FMA, the sum's
// by TwoSum
__device__ __forceinline__ void ff_mul_acc(float& hi, float& lo, float z, float w_hi, float w_lo) {
  const float p = __fmul_rn(z, w_hi);
  const float e = __fmaf_rn(z, w_hi, -p);
  two_sum_acc(hi, lo, p);
  lo = __fadd_rn(lo, __fmaf_rn(z, w_lo, e));
}

// The block's sums of v[0..N) (per thread values), in a fixed order; valid
// in thread 0.  red holds kMbFftThreads / 32 doubles per value.
template <int N>
__device__ __forceinline__ void block_sums(double* v, double (*red)[kMbFftThreads / 32]) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int n = 0; n < N; ++n) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v[n] += __shfl_xor_sync(0xffffffffu, v[n], o);
    if (lane == 0) red[n][warp] = v[n];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int n = 0; n < N; ++n) {
      double t = 0.0;
      for (int w = 0; w < kMbFftThreads / 32; ++w) t += red[n][w];
      v[n] = t;
    }
  }
}

// The work items of a launch: every (point, detector pair), or, with a list,
// the listed points' pairs.
__device__ __forceinline__ int64_t mb_fft_items(const LaunchArgs& a, const MbFftBand& bd, int P) {
  return bd.list ? (int64_t)(*bd.list_count) * P : a.B * P;
}

template <int D>
__global__ void __launch_bounds__(kMbFftThreads) k_mb_hh_fft(LaunchArgs a, MbFftBand bd, double2* scratch) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ double red[2][kMbFftThreads / 32];
  const int log2m = bd.log2m, sh = bd.log2m_max;
  const uint32_t M = 1u << log2m, half = M >> 1;
  double2* buf = bd.in_smem ? reinterpret_cast<double2*>(smem_raw) : scratch + (size_t)blockIdx.x * M;
  constexpr int P = (D + 1) / 2;
  const int64_t n_items = mb_fft_items(a, bd, P);
  const int64_t k_b = a.mb_band_start[bd.band], nk = a.mb_band_start[bd.band + 1] - k_b;
  const bool tf2 = a.model == GWL_MODEL_TAYLORF2;
  for (int64_t item = blockIdx.x; item < n_items; item += gridDim.x) {
    const int64_t slot = item / P;
    const int64_t i = bd.list ? (int64_t)bd.list[slot] : slot;
    const int d1 = 2 * (int)(item - slot * P), d2 = d1 + 1;  // d2 == D: no partner
    const PointRec& r = a.rec[i];
    for (uint32_t q = threadIdx.x; q < M; q += blockDim.x) buf[q] = make_double2(0.0, 0.0);
    __syncthreads();
    // ---- C at the band's bins and their mirror images --------------------
    if (r.valid) {
      const double u = tf2 ? cbrt(kPi * r.m_sec) : 0.0, lnu = tf2 ? log(u) : 0.0;
      const double pu5 = tf2 ? 3.0 / (128.0 * r.eta) / (u * u * u * u * u) : 0.0;
      for (int64_t t = threadIdx.x; t < nk; t += blockDim.x) {
        const int64_t k = k_b + t;
        const double f = a.mb_freq[k];
        double2 hp = make_double2(0.0, 0.0), hx = make_double2(0.0, 0.0);
        if (!(tf2 ? tf2_pols_t(a, r, a.mb_pow[k], f, u, lnu, pu5, hp, hx) : plain_pols(a, r, f, hp, hx))) continue;
        const double sw = bd.sqrtw[k];
        double2 w[2] = {make_double2(0.0, 0.0), make_double2(0.0, 0.0)};
#pragma unroll
        for (int e = 0; e < 2; ++e) {
          const int d = d1 + e;
          if (d >= D) break;
          // interferometer.py:341-362 at explicit frequencies (no mask)
          const double sre = hp.x * r.fp[d] + hx.x * r.fx[d], sim = hp.y * r.fp[d] + hx.y * r.fx[d];
          double sn, cs;
          sincos(2.0 * kPi * r.dt[d] * f, &sn, &cs);
          w[e] = make_double2(sw * (sre * cs + sim * sn), sw * (sim * cs - sre * sn));
        }
        const uint32_t m = (uint32_t)(bd.ks + t);  // 1 <= m < M / 2 (checked on the host)
        if (!GWL_INDEX_OK((int64_t)m - 1, half - 1, a.status)) continue;
        buf[m] = make_double2(w[0].x - w[1].y, w[0].y + w[1].x);
        buf[M - m] = make_double2(w[0].x + w[1].y, w[1].x - w[0].y);
      }
    }
    __syncthreads();
    packed_transform<double>(buf, log2m, nullptr, 0, bd.tw, sh);
    // ---- odd bins: sum_j |Z_j|^2 Re I_2j+1 per detector --------------------
    const double* o1 = bd.odd[d1];
    const double* o2 = d2 < D ? bd.odd[d2] : nullptr;
    double v[2] = {0.0, 0.0};
    for (uint32_t j = threadIdx.x; j < half; j += blockDim.x) {
      const double2 F = buf[j], R = buf[M - 1 - j];
      const double ax = F.x + R.x, ay = F.y - R.y;  // 2 Z_d1
      v[0] += (ax * ax + ay * ay) * o1[j];
      if (o2) {
        const double bx = F.y + R.y, by = F.x - R.x;  // 2 i Z_d2 up to sign
        v[1] += (bx * bx + by * by) * o2[j];
      }
    }
    block_sums<2>(v, red);
    if (threadIdx.x == 0) {
      double* out = bd.out + (int64_t)bd.band * D * a.B;
      out[(int64_t)d1 * a.B + i] = 0.25 * bd.scale * v[0];
      if (d2 < D) out[(int64_t)d2 * a.B + i] = 0.25 * bd.scale * v[1];
    }
    // the next item's zeroing of buf follows block_sums' barrier, and red is
    // written again only after several more barriers
  }
}

// Mixed precision (TaylorF2): the banded values in float32 from the exact
// fixed-point phase, float32 transforms, float-float sums and the error
// bound.  At most 64 registers (two 512-thread CTAs per SM).
template <int D>
__global__ void __launch_bounds__(kMbFftThreads, 2) k_mb_hh_fft32(LaunchArgs a, MbFftBand bd, float2* scratch) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ double red[6][kMbFftThreads / 32];
  __shared__ uint64_t s_yx[4];        // Y, X of the pair's detectors (0.64 fixed point)
  __shared__ int64_t s_kb[2];         // the point's band [f_min, f_isco) among the banded frequencies
  const int log2m = bd.log2m, sh = bd.log2m_max;
  const uint32_t M = 1u << log2m, half = M >> 1;
  float2* buf = bd.in_smem ? reinterpret_cast<float2*>(smem_raw) : scratch + (size_t)blockIdx.x * M;
  constexpr int P = (D + 1) / 2;
  const int64_t n_items = a.B * P;
  const int64_t k_b = a.mb_band_start[bd.band], nk = a.mb_band_start[bd.band + 1] - k_b;
  for (int64_t item = blockIdx.x; item < n_items; item += gridDim.x) {
    const int64_t i = item / P;
    const int d1 = 2 * (int)(item - i * P), d2 = d1 + 1;  // d2 == D: no partner
    const PointRec& r = a.rec[i];
    for (uint32_t q = threadIdx.x; q < M; q += blockDim.x) buf[q] = make_float2(0.f, 0.f);
    if (r.valid && threadIdx.x < 2) {
      // detector d's shift in this band, 0.64 fixed point (as the mixed
      // multi-banding kernel forms it)
      const int d = d1 + (int)threadIdx.x;
      uint64_t Y = 0, X = 0;
      if (d < D) {
        const double dt = r.dt[d];
        const double y = a.mb_freq[k_b] * dt, x = a.mb_band_df[bd.band] * dt;
        double fy = ldexp(y - floor(y), 64), fx = ldexp(x - floor(x), 64);
        if (!(fy < 18446744073709551616.0)) fy = 0.0;
        if (!(fx < 18446744073709551616.0)) fx = 0.0;
        Y = (uint64_t)fy;
        X = (uint64_t)fx;
      }
      s_yx[2 * threadIdx.x] = Y;
      s_yx[2 * threadIdx.x + 1] = X;
    }
    if (r.valid && threadIdx.x == 32) {
      int64_t lo = 0, hi = a.mb_points;
      while (lo < hi) {
        const int64_t mid = (lo + hi) / 2;
        if (a.mb_freq[mid] >= a.fmin) hi = mid; else lo = mid + 1;
      }
      s_kb[0] = lo;
      hi = a.mb_points;
      while (lo < hi) {
        const int64_t mid = (lo + hi) / 2;
        if (a.mb_freq[mid] >= r.f_isco) hi = mid; else lo = mid + 1;
      }
      s_kb[1] = lo;
    }
    __syncthreads();
    if (r.valid) {
      float ch[kNumBasis + 1], cl[kNumBasis + 1];
#pragma unroll
      for (int b = 0; b <= kNumBasis; ++b) {
        ch[b] = r.c_hi[b];
        cl[b] = r.c_lo[b];
      }
      // Q_d = Fp (1 + c^2) / 2 - i Fx c of the pair's detectors
      const double ci = r.cos_i, pfac = (1.0 + ci * ci) / 2.0;
      const float q1r = (float)(r.fp[d1] * pfac), q1i = (float)(-r.fx[d1] * ci);
      const float q2r = d2 < D ? (float)(r.fp[d2] * pfac) : 0.f, q2i = d2 < D ? (float)(-r.fx[d2] * ci) : 0.f;
      const uint64_t Y1 = s_yx[0], X1 = s_yx[1], Y2 = s_yx[2], X2 = s_yx[3];
      const int64_t kb0 = s_kb[0], kb1 = s_kb[1];
      for (int64_t t = threadIdx.x; t < nk; t += blockDim.x) {
        const int64_t k = k_b + t;
        if (k < kb0 || k >= kb1) continue;
        const float4* bp = reinterpret_cast<const float4*>(a.mb_basis + k * kNumBasis);
        float s_hi = ch[kNumBasis], s_lo = cl[kNumBasis];
#pragma unroll
        for (int q = 0; q < kNumBasis / 2; ++q) {
          const float4 v = __ldg(bp + q);
          ff_mac(s_hi, s_lo, ch[2 * q], cl[2 * q], v.x, v.y);
          ff_mac(s_hi, s_lo, ch[2 * q + 1], cl[2 * q + 1], v.z, v.w);
        }
        const uint64_t base = to_fixed(s_hi, s_lo);
        const float amp = __ldg(bd.aw + k);
        float w1r, w1i, w2r = 0.f, w2i = 0.f;
        {
          const uint32_t top = (uint32_t)((base + Y1 + (uint64_t)t * X1 + 0x80000000ull) >> 32);
          float sn, cs;
          sincospif(__fmul_rn(__int2float_rn((int)top), 4.656612873077393e-10f), &sn, &cs);
          // Q amp (cos - i sin)
          const float er = amp * cs, ei = -amp * sn;
          w1r = q1r * er - q1i * ei;
          w1i = q1r * ei + q1i * er;
        }
        if (d2 < D) {
          const uint32_t top = (uint32_t)((base + Y2 + (uint64_t)t * X2 + 0x80000000ull) >> 32);
          float sn, cs;
          sincospif(__fmul_rn(__int2float_rn((int)top), 4.656612873077393e-10f), &sn, &cs);
          const float er = amp * cs, ei = -amp * sn;
          w2r = q2r * er - q2i * ei;
          w2i = q2r * ei + q2i * er;
        }
        const uint32_t m = (uint32_t)(bd.ks + t);  // 1 <= m < M / 2 (checked on the host)
        if (!GWL_INDEX_OK((int64_t)m - 1, half - 1, a.status)) continue;
        buf[m] = make_float2(w1r - w2i, w1i + w2r);
        buf[M - m] = make_float2(w1r + w2i, w2r - w1i);
      }
    }
    __syncthreads();
    packed_transform<float>(buf, log2m, bd.in_smem ? nullptr : reinterpret_cast<float2*>(smem_raw),
                            kMbFft32BlockLog2, bd.tw32, sh);
    // ---- odd bins: sum |2Z|^2 o per detector in float-float (the weights as
    // float-float pairs, scaled by the band's largest), and in float the
    // norms of the error bound, sum |2Z|^2 o^2 and sum |2Z|^2 --------------
    const float2* o1 = bd.odd32[d1];
    const float2* o2 = d2 < D ? bd.odd32[d2] : nullptr;
    float sh1 = 0.f, sl1 = 0.f, sh2 = 0.f, sl2 = 0.f, n1 = 0.f, m1 = 0.f, n2 = 0.f, m2 = 0.f;
    for (uint32_t j = threadIdx.x; j < half; j += blockDim.x) {
      const float2 F = buf[j], R = buf[M - 1 - j];
      const float ax = F.x + R.x, ay = F.y - R.y;  // 2 Z_d1
      const float z1 = __fmaf_rn(ax, ax, __fmul_rn(ay, ay));
      const float2 w1 = o1[j];
      ff_mul_acc(sh1, sl1, z1, w1.x, w1.y);
      n1 = __fmaf_rn(__fmul_rn(z1, w1.x), w1.x, n1);
      m1 = __fadd_rn(m1, z1);
      if (o2) {
        const float bx = F.y + R.y, by = F.x - R.x;  // 2 i Z_d2 up to sign
        const float z2 = __fmaf_rn(bx, bx, __fmul_rn(by, by));
        const float2 w2 = o2[j];
        ff_mul_acc(sh2, sl2, z2, w2.x, w2.y);
        n2 = __fmaf_rn(__fmul_rn(z2, w2.x), w2.x, n2);
        m2 = __fadd_rn(m2, z2);
      }
    }
    double v[6] = {(double)sh1 + (double)sl1, (double)n1, (double)m1, (double)sh2 + (double)sl2, (double)n2,
                   (double)m2};
    block_sums<6>(v, red);
    if (threadIdx.x == 0) {
      // <h|h> scale: the point's amplitude squared times the table's scale squared
      const double g = 0.25 * bd.scale * (r.valid ? r.amp * r.amp : 0.0) * bd.aw_scale * bd.aw_scale;
      const double gs = g * bd.odd32_scale;  // the float weights are o / odd32_scale
      const double eta = kFft32Err * kU32 * sqrt((double)(log2m + 2));
      const int64_t o = (int64_t)bd.band * D * a.B;
      bd.out[o + (int64_t)d1 * a.B + i] = gs * v[0];
      // |d lnL| <= |d <h|h>| / 2: the lnL's slope in <h|h> is -1/2 without
      // the distance table (with it the host keeps the float64 transforms)
      bd.err[o + (int64_t)d1 * a.B + i] = 0.5 * gs * eta * sqrt(v[1]) * sqrt(v[2]);
      if (d2 < D) {
        bd.out[o + (int64_t)d2 * a.B + i] = gs * v[3];
        bd.err[o + (int64_t)d2 * a.B + i] = 0.5 * gs * eta * sqrt(v[4]) * sqrt(v[5]);
      }
    }
  }
}

// The points whose float32 odd-bin error, summed over bands >= 1 and
// detectors, exceeds the tolerance: listed (in any order) for the float64
// kernel.
__global__ void k_mb_fft_marks(LaunchArgs a, const double* err, double tol, int32_t* list, int32_t* count) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.B) return;
  double e = 0.0;
  for (int b = 1; b < a.mb_bands; ++b)
    for (int d = 0; d < a.n_det; ++d) e += err[((int64_t)b * a.n_det + d) * a.B + i];
  if (!(e <= tol)) list[atomicAdd(count, 1)] = (int32_t)i;
}

template <int D>
cudaError_t launch_d(const LaunchArgs& a, const MbFftBand& bd, void* scratch, int64_t scratch_slots, bool mixed,
                     cudaStream_t s) {
  constexpr int P = (D + 1) / 2;
  const int64_t n_items = a.B * P;  // a list never holds more
  if (n_items <= 0) return cudaSuccess;
  // shared memory: the whole transform, or (float32, global slots) one block of it
  const size_t smem = bd.in_smem ? (mixed ? sizeof(float2) : sizeof(double2)) << bd.log2m
                                 : (mixed ? sizeof(float2) << kMbFft32BlockLog2 : 0);
  int64_t grid = n_items;
  if (!bd.in_smem) grid = std::min<int64_t>(n_items, scratch_slots);
  if (grid <= 0) return cudaErrorInvalidValue;
  if (mixed) {
    if (smem > 48 * 1024) cudaFuncSetAttribute(k_mb_hh_fft32<D>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_mb_hh_fft32<D><<<(unsigned)grid, kMbFftThreads, smem, s>>>(a, bd, static_cast<float2*>(scratch));
  } else {
    if (smem > 48 * 1024) cudaFuncSetAttribute(k_mb_hh_fft<D>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_mb_hh_fft<D><<<(unsigned)grid, kMbFftThreads, smem, s>>>(a, bd, static_cast<double2*>(scratch));
  }
  return cudaGetLastError();
}

}  // namespace

size_t mb_hh_fft_smem(int log2m) {
  const size_t bytes = sizeof(double2) << log2m;
  return log2m <= kMbFftSmemLog2 ? bytes : 0;
}

bool mb_hh_fft32_in_smem(int log2m) { return log2m <= kMbFft32SmemLog2; }

cudaError_t launch_mb_hh_fft(const LaunchArgs& a, const MbFftBand& bd, void* scratch, int64_t scratch_slots,
                             bool mixed, cudaStream_t s) {
  switch (a.n_det) {
    case 1: return launch_d<1>(a, bd, scratch, scratch_slots, mixed, s);
    case 2: return launch_d<2>(a, bd, scratch, scratch_slots, mixed, s);
    case 3: return launch_d<3>(a, bd, scratch, scratch_slots, mixed, s);
    default: return launch_d<4>(a, bd, scratch, scratch_slots, mixed, s);
  }
}

cudaError_t launch_mb_fft_marks(const LaunchArgs& a, const double* err, double tol, int32_t* list, int32_t* count,
                                cudaStream_t s) {
  const int threads = 256;
  k_mb_fft_marks<<<(unsigned)((a.B + threads - 1) / threads), threads, 0, s>>>(a, err, tol, list, count);
  return cudaGetLastError();
}

}  // namespace gwl
