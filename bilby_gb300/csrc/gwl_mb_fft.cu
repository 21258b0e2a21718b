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
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>

#include "gwl_device.cuh"
#include "gwl_internal.h"
#include "gwl_marg_common.cuh"
#include "gwl_math.cuh"

namespace gwl {

namespace {

constexpr int kMbFftThreads = 512;

template <int D>
__global__ void __launch_bounds__(kMbFftThreads) k_mb_hh_fft(LaunchArgs a, MbFftBand bd, double2* scratch) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ double red[2][kMbFftThreads / 32];
  const int log2m = bd.log2m, sh = bd.log2m_max;
  const uint32_t M = 1u << log2m, half = M >> 1;
  double2* buf = bd.in_smem ? reinterpret_cast<double2*>(smem_raw) : scratch + (size_t)blockIdx.x * M;
  constexpr int P = (D + 1) / 2;
  const int64_t n_items = a.B * P;
  const int64_t k_b = a.mb_band_start[bd.band], nk = a.mb_band_start[bd.band + 1] - k_b;
  const bool tf2 = a.model == GWL_MODEL_TAYLORF2;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int64_t item = blockIdx.x; item < n_items; item += gridDim.x) {
    const int64_t i = item / P;
    const int d1 = 2 * (int)(item - i * P), d2 = d1 + 1;  // d2 == D: no partner
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
    // ---- inverse DFT, decimation in frequency ----------------------------
    // radix-4 passes, each two radix-2 stages (half-sizes h and q = h / 2) on
    // {x0, x1, x2, x3} at i0 + {0, q, 2q, 3q} with W = exp(i pi j / h):
    //   z0 = (x0 + x2) + (x1 + x3)      z1 = W^2 ((x0 + x2) - (x1 + x3))
    //   z2 = W ((x0 - x2) + i (x1 - x3))  z3 = W^3 ((x0 - x2) - i (x1 - x3))
    // then, for odd log2 M, the radix-2 stage h = 1
    int lh = log2m - 1;
    for (; lh >= 1; lh -= 2) {
      const int lq = lh - 1;
      const uint32_t q = 1u << lq;
      for (uint32_t t = threadIdx.x; t < (M >> 2); t += blockDim.x) {
        const uint32_t j = t & (q - 1), i0 = ((t >> lq) << (lq + 2)) + j;
        const double2 x0 = buf[i0], x1 = buf[i0 + q], x2 = buf[i0 + 2 * q], x3 = buf[i0 + 3 * q];
        const int s = sh - lh;
        const double2 w1 = bd.tw[(size_t)j << s], w2 = bd.tw[(size_t)(2 * j) << s], w3 = bd.tw[(size_t)(3 * j) << s];
        const double ar = x0.x + x2.x, ai = x0.y + x2.y, br = x1.x + x3.x, bi = x1.y + x3.y;
        const double cr = x0.x - x2.x, ci = x0.y - x2.y, dr = x1.x - x3.x, di = x1.y - x3.y;
        buf[i0] = make_double2(ar + br, ai + bi);
        const double er = ar - br, ei = ai - bi;        // times conj(w2)
        buf[i0 + q] = make_double2(er * w2.x + ei * w2.y, ei * w2.x - er * w2.y);
        const double fr = cr - di, fi = ci + dr;        // (x0 - x2) + i (x1 - x3), times conj(w1)
        buf[i0 + 2 * q] = make_double2(fr * w1.x + fi * w1.y, fi * w1.x - fr * w1.y);
        const double gr = cr + di, gi = ci - dr;        // (x0 - x2) - i (x1 - x3), times conj(w3)
        buf[i0 + 3 * q] = make_double2(gr * w3.x + gi * w3.y, gi * w3.x - gr * w3.y);
      }
      __syncthreads();
    }
    if (lh == 0) {
      for (uint32_t t = threadIdx.x; t < half; t += blockDim.x) {
        const double2 x0 = buf[2 * t], x1 = buf[2 * t + 1];
        buf[2 * t] = make_double2(x0.x + x1.x, x0.y + x1.y);
        buf[2 * t + 1] = make_double2(x0.x - x1.x, x0.y - x1.y);
      }
      __syncthreads();
    }
    // ---- times exp(-i pi n / M) / M at bit-reversed position of n --------
    const double inv_m = ldexp(1.0, -log2m);
    for (uint32_t q = threadIdx.x; q < M; q += blockDim.x) {
      const uint32_t n = __brev(q) >> (32 - log2m);
      const double2 w = bd.tw[(size_t)n << (sh - log2m)];
      const double2 x = buf[q];
      buf[q] = make_double2((x.x * w.x - x.y * w.y) * inv_m, (x.x * w.y + x.y * w.x) * inv_m);
    }
    __syncthreads();
    // ---- forward DFT, decimation in time ---------------------------------
    // for odd log2 M the radix-2 stage h = 1 first, then radix-4 passes, each
    // two radix-2 stages (h and 2h) on {x0, x1, x2, x3} at i0 + {0, h, 2h, 3h}
    // with U = exp(-i pi j / 2h), a = x0, b = U^2 x1, c = U x2, d = U^3 x3:
    //   z0 = (a + b) + (c + d)    z2 = (a + b) - (c + d)
    //   z1 = (a - b) - i (c - d)  z3 = (a - b) + i (c - d)
    lh = 0;
    if (log2m & 1) {
      for (uint32_t t = threadIdx.x; t < half; t += blockDim.x) {
        const double2 x0 = buf[2 * t], x1 = buf[2 * t + 1];
        buf[2 * t] = make_double2(x0.x + x1.x, x0.y + x1.y);
        buf[2 * t + 1] = make_double2(x0.x - x1.x, x0.y - x1.y);
      }
      __syncthreads();
      lh = 1;
    }
    for (; lh + 1 < log2m; lh += 2) {
      const uint32_t h = 1u << lh;
      for (uint32_t t = threadIdx.x; t < (M >> 2); t += blockDim.x) {
        const uint32_t j = t & (h - 1), i0 = ((t >> lh) << (lh + 2)) + j;
        const double2 x0 = buf[i0], x1 = buf[i0 + h], x2 = buf[i0 + 2 * h], x3 = buf[i0 + 3 * h];
        const int s = sh - lh - 1;
        const double2 u1 = bd.tw[(size_t)j << s], u2 = bd.tw[(size_t)(2 * j) << s], u3 = bd.tw[(size_t)(3 * j) << s];
        const double br = x1.x * u2.x - x1.y * u2.y, bi = x1.x * u2.y + x1.y * u2.x;
        const double cr = x2.x * u1.x - x2.y * u1.y, ci = x2.x * u1.y + x2.y * u1.x;
        const double dr = x3.x * u3.x - x3.y * u3.y, di = x3.x * u3.y + x3.y * u3.x;
        const double pr = x0.x + br, pi = x0.y + bi, mr = x0.x - br, mi = x0.y - bi;
        const double sr = cr + dr, si = ci + di, tr = cr - dr, ti = ci - di;
        buf[i0] = make_double2(pr + sr, pi + si);
        buf[i0 + 2 * h] = make_double2(pr - sr, pi - si);
        buf[i0 + h] = make_double2(mr + ti, mi - tr);      // (a - b) - i (c - d)
        buf[i0 + 3 * h] = make_double2(mr - ti, mi + tr);  // (a - b) + i (c - d)
      }
      __syncthreads();
    }
    // ---- odd bins: sum_j |Z_j|^2 Re I_2j+1 per detector --------------------
    const double* o1 = bd.odd[d1];
    const double* o2 = d2 < D ? bd.odd[d2] : nullptr;
    double s1 = 0.0, s2 = 0.0;
    for (uint32_t j = threadIdx.x; j < half; j += blockDim.x) {
      const double2 F = buf[j], R = buf[M - 1 - j];
      const double ax = F.x + R.x, ay = F.y - R.y;  // 2 Z_d1
      s1 += (ax * ax + ay * ay) * o1[j];
      if (o2) {
        const double bx = F.y + R.y, by = F.x - R.x;  // 2 i Z_d2 up to sign
        s2 += (bx * bx + by * by) * o2[j];
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      s1 += __shfl_xor_sync(0xffffffffu, s1, o);
      s2 += __shfl_xor_sync(0xffffffffu, s2, o);
    }
    if (lane == 0) {
      red[0][warp] = s1;
      red[1][warp] = s2;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      double t1 = 0.0, t2 = 0.0;
      for (int w = 0; w < kMbFftThreads / 32; ++w) {
        t1 += red[0][w];
        t2 += red[1][w];
      }
      double* out = bd.out + (int64_t)bd.band * D * a.B;
      out[(int64_t)d1 * a.B + i] = 0.25 * bd.scale * t1;
      if (d2 < D) out[(int64_t)d2 * a.B + i] = 0.25 * bd.scale * t2;
    }
    // the next item's zeroing of buf follows the barrier above, and red is
    // written again only after several more barriers
  }
}

}  // namespace

size_t mb_hh_fft_smem(int log2m) {
  const size_t bytes = sizeof(double2) << log2m;
  return log2m <= kMbFftSmemLog2 ? bytes : 0;
}

int mb_hh_fft_threads() { return kMbFftThreads; }

cudaError_t launch_mb_hh_fft(const LaunchArgs& a, const MbFftBand& bd, double2* scratch, int64_t scratch_slots,
                             cudaStream_t s) {
  const int P = (a.n_det + 1) / 2;
  const int64_t n_items = a.B * P;
  if (n_items <= 0) return cudaSuccess;
  const size_t smem = bd.in_smem ? mb_hh_fft_smem(bd.log2m) : 0;
  int64_t grid = n_items;
  if (!bd.in_smem) grid = std::min<int64_t>(n_items, scratch_slots);
  if (grid <= 0) return cudaErrorInvalidValue;
  switch (a.n_det) {
    case 1:
      if (smem > 48 * 1024) cudaFuncSetAttribute(k_mb_hh_fft<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      k_mb_hh_fft<1><<<(unsigned)grid, kMbFftThreads, smem, s>>>(a, bd, scratch);
      break;
    case 2:
      if (smem > 48 * 1024) cudaFuncSetAttribute(k_mb_hh_fft<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      k_mb_hh_fft<2><<<(unsigned)grid, kMbFftThreads, smem, s>>>(a, bd, scratch);
      break;
    case 3:
      if (smem > 48 * 1024) cudaFuncSetAttribute(k_mb_hh_fft<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      k_mb_hh_fft<3><<<(unsigned)grid, kMbFftThreads, smem, s>>>(a, bd, scratch);
      break;
    default:
      if (smem > 48 * 1024) cudaFuncSetAttribute(k_mb_hh_fft<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      k_mb_hh_fft<4><<<(unsigned)grid, kMbFftThreads, smem, s>>>(a, bd, scratch);
      break;
  }
  return cudaGetLastError();
}

}  // namespace gwl
