// Time marginalisation (bilby/gw/likelihood/base.py:325-330, 794-820,
// 1027-1035), composed with phase (ln I0) and distance (bicubic table)
// marginalisation.
//
// One CTA per parameter point:
//   A. the fused integrand z_k = 4/T sum_det h_det,k conj(d_k) / S_k for
//      k < L = n_bins - 1, written in bit-reversed order into shared memory
//      (mixed precision, float32) or into this CTA's slot of an L2-resident
//      work buffer (float64; 16 B * L does not fit in shared memory);
//   B. an in-place radix-2 decimation-in-time FFT of length L (numpy's sign
//      convention, exp(-2 pi i m k / L)).  For L = m 2^p with m odd and
//      greater than one, the integrand's residue class r = k mod m goes to
//      block r of the buffer (bit-reversed there), the radix-2 stages run as m
//      independent transforms Y_r of length N = 2^p, and the output is
//      X[j] = sum_r exp(-2 pi i r j / L) Y_r[j mod N], formed only where it is
//      read (the prior window's samples; every j for the float64 series);
//   C. the time samples inside the geocent_time prior, paired with FFT index
//      j exactly as the reference pairs them (times[j] = start + (j+1) 2/fs
//      + jitter), the per-sample marginalised log-likelihood, and a
//      logsumexp weighted by prior(t_j) * delta_tc, reduced in a fixed order.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <map>
#include <mutex>

#include "gwl_device.cuh"
#include "gwl_device_cache.h"
#include "gwl_internal.h"
#include "gwl_marg_common.cuh"
#include "gwl_math.cuh"
#include "gwl_phase.cuh"

namespace gwl {

constexpr int kTmThreads = 512;
constexpr int kTmTwiddleRows = 128;
// Error model of the mixed TaylorF2 kernel (|dlnL| <= s |dX| over the prior
// window, s from tm_sensitivity): __sincosf's and the weights' independent
// per-bin errors and the float32 transform's rounding as ||z||_2 where the
// outputs are noise, the transform's coherent rounding as |X| at a peak.
// Measured on tf2_marg_8s (8192 prior draws and loud templates at 20-800 Mpc
// with |X| up to 3e4): |dX| <= 2e-6 ||z||_2 + 1.3e-7 |X|max; the per-sample
// lnL in float32 adds one rounding of about 6e-8 |X|.
constexpr double kTmErrNorm = 2e-6;
constexpr double kTmErrPeak = 3e-7;

// Block-wide reductions over kTmThreads threads in a fixed tree order.
__device__ double block_max(double v, double* red) {
  red[threadIdx.x] = v;
  __syncthreads();
  for (int s = kTmThreads / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + s]);
    __syncthreads();
  }
  const double r = red[0];
  __syncthreads();
  return r;
}

__device__ double block_sum(double v, double* red) {
  red[threadIdx.x] = v;
  __syncthreads();
  for (int s = kTmThreads / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] = red[threadIdx.x] + red[threadIdx.x + s];
    __syncthreads();
  }
  const double r = red[0];
  __syncthreads();
  return r;
}

template <int D, bool MIXED>
__global__ void __launch_bounds__(kTmThreads) k_time_marg(LaunchArgs a, const typename TmTypes<MIXED>::C* twiddle,
                                                          int log2N, int m_odd) {
  using C = typename TmTypes<MIXED>::C;
  using R = typename TmTypes<MIXED>::R;
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ double red[2 * kTmThreads];
  __shared__ float s_coef[2 * kMaxDet];
  __shared__ double s_scal[6];
  __shared__ long long s_jr[2];
  __shared__ SplineRowF s_row;
  // mixed: the FFT twiddles exp(-2 pi i q / L), q < L / 2, as products of two
  // shared-memory tables (q = 128 q1 + q2), instead of loads from global memory
  __shared__ float2 tw_hi[kTmTwiddleRows], tw_lo[kTmTwiddleRows];
  __shared__ float2 s_w16[16];
  const int64_t L = a.n_fft, N2 = (int64_t)1 << log2N;  // L = m_odd N2
  const double norm = 4.0 / a.duration;
  // buffer position of integrand bin k: block k mod m_odd, bit-reversed within it
  const auto brpos = [&](int64_t k) -> int64_t {
    if (m_odd == 1) return (int64_t)bit_reverse((uint32_t)k, log2N);
    return (k % m_odd) * N2 + (int64_t)bit_reverse((uint32_t)(k / m_odd), log2N);
  };
  if constexpr (MIXED) {
    const int64_t half = L / 2;
    for (int q = threadIdx.x; q < kTmTwiddleRows; q += blockDim.x) {
      const int64_t qh = (int64_t)q * kTmTwiddleRows;
      tw_hi[q] = qh < half ? reinterpret_cast<const float2*>(twiddle)[qh] : make_float2(1.f, 0.f);
      tw_lo[q] = q < half ? reinterpret_cast<const float2*>(twiddle)[q] : make_float2(1.f, 0.f);
    }
    // the 16th roots of unity exp(-2 pi i m / 16) (the table holds q < L / 2)
    if (threadIdx.x < 8) {
      const float2 t = reinterpret_cast<const float2*>(twiddle)[(int64_t)threadIdx.x * (L / 16)];
      s_w16[threadIdx.x] = t;
      s_w16[threadIdx.x + 8] = make_float2(-t.x, -t.y);
    }
    __syncthreads();
  }
  // mixed: the distance spline's knots in shared memory, after the FFT buffer
  float* s_tx = reinterpret_cast<float*>(smem + (MIXED ? (L + L / 16) * sizeof(float2) : 0));
  float* s_ty = s_tx + a.nx;
  if (MIXED && a.dist_marg) {
    for (int q = threadIdx.x; q < a.nx; q += blockDim.x) s_tx[q] = a.tx_f[q];
    for (int q = threadIdx.x; q < a.ny; q += blockDim.x) s_ty[q] = a.ty_f[q];
    __syncthreads();
  }
  const auto tw = [&](int64_t q) -> C {
    if constexpr (MIXED) {
      const float2 h = tw_hi[q / kTmTwiddleRows], l = tw_lo[q % kTmTwiddleRows];
      C w;
      w.x = h.x * l.x - h.y * l.y;
      w.y = h.x * l.y + h.y * l.x;
      return w;
    } else {
      return twiddle[q];
    }
  };
  // mixed: one padding slot after every 16 elements of the shared-memory
  // buffer, so that the strided accesses of the FFT passes spread over the banks
  const auto P = [](int64_t q) -> int64_t { return MIXED ? q + (q >> 4) : q; };
  // output j of the length-L transform from the m_odd blocks' transforms
  const auto out_at = [&](const C* b, int64_t j) -> C {
    const int64_t jn = j & (N2 - 1);
    if (m_odd == 1) return b[P(jn)];
    C x;
    x.x = 0;
    x.y = 0;
    int64_t q = 0;  // r j mod L
    for (int r = 0; r < m_odd; ++r) {
      C w = q < L / 2 ? tw(q) : tw(q - L / 2);
      if (q >= L / 2) {
        w.x = -w.x;
        w.y = -w.y;
      }
      const C y = b[P(r * N2 + jn)];
      x.x += w.x * y.x - w.y * y.y;
      x.y += w.x * y.y + w.y * y.x;
      q += j;
      if (q >= L) q -= L;
    }
    return x;
  };
  for (int64_t i = blockIdx.x; i < a.B; i += gridDim.x) {
    C* buf = MIXED ? reinterpret_cast<C*>(smem) : reinterpret_cast<C*>(a.tm_work) + (size_t)blockIdx.x * L;
    const PointRec& r = a.rec[i];
    // ---- A: integrand --------------------------------------------------
    // (multi-banding with the IFFT-FFT <h|h>: its odd-bin part, once)
    double hh_part = threadIdx.x == 0 ? mb_fft_hh_total(a, i) : 0.0;
    float z2 = 0.f;  // mixed TaylorF2: sum of |z_k|^2 over this thread's bins (error bound)
    if constexpr (MIXED) {
      // per-point float32 coefficients, computed by the float64 prologue
      if (threadIdx.x < 2 * D) s_coef[threadIdx.x] = r.tm_coef[threadIdx.x];
      __syncthreads();
      float gre[D], gim[D], cre[D], cim[D];
      uint32_t xl[D], xh[D];
      float ch[kNumBasis + 1], cl[kNumBasis + 1];
      for (int d = 0; d < D; ++d) {
        xl[d] = r.xfix[d][0];
        xh[d] = r.xfix[d][1];
        gre[d] = cre[d] = s_coef[2 * d];
        gim[d] = cim[d] = s_coef[2 * d + 1];
      }
      for (int b = 0; b <= kNumBasis; ++b) {
        ch[b] = r.c_hi[b];
        cl[b] = r.c_lo[b];
      }
      const float f0h = (float)r.sg_f0, f0l = (float)(r.sg_f0 - (double)f0h);
      const float gah = (float)r.sg_a, gal = (float)(r.sg_a - (double)gah);
      if (a.model == GWL_MODEL_TAYLORF2) {
        // The integrand fused with the first four FFT stages.  After them the
        // positions 16 b .. 16 b + 15 hold the 16-point DFT of the bins
        // q + j L/16 (j < 16), q = bitrev(b) over log2(L) - 4 bits.  The band
        // holds a few thousand of the L bins, so a residue q has 0-3 of its 16
        // bins in it: a thread takes blocks b, evaluates their in-band bins,
        // and writes the 16 outputs (zeros when none); consecutive threads
        // write consecutive blocks.
        const int64_t R = L >> 4, R2 = N2 >> 4;
        const int lr = log2N - 4;
        const int64_t ks = max(r.k_start, a.k_lo), ke = min(min(r.k_end, a.k_hi), L);
        const float4* basis4 = reinterpret_cast<const float4*>(a.basis);
        // ceil(x / R) for 0 < x < 2^32 (R = m_odd 2^lr: a shift when m_odd = 1),
        // in 32-bit arithmetic
        const auto cdiv_R = [&](int64_t x) -> int {
          const uint32_t n = (uint32_t)x + (uint32_t)R - 1u;
          return (int)(m_odd == 1 ? n >> lr : n / (uint32_t)R);
        };
        for (int64_t bb = threadIdx.x; bb < R; bb += blockDim.x) {
          // block bb / R2 of the m_odd transforms: bins q + j L / 16 with
          // q = (bb / R2) + m_odd bitrev(bb mod R2), R2 = 2^lr
          const int64_t q = (bb >> lr) + m_odd * (int64_t)bit_reverse((uint32_t)(bb & (R2 - 1)), lr);
          float yr[16], yi[16];
#pragma unroll
          for (int v = 0; v < 16; ++v) yr[v] = yi[v] = 0.f;
          // in-band j: ks <= q + j R < ke
          const int j0 = r.valid ? (ks > q ? cdiv_R(ks - q) : 0) : 16;
          const int j1 = r.valid ? (ke > q ? min(16, cdiv_R(ke - q)) : 0) : 0;
          for (int j = j0; j < j1; ++j) {
            const int64_t k = q + (int64_t)j * R;
            float s_hi = ch[kNumBasis], s_lo = cl[kNumBasis];
#pragma unroll
            for (int qq = 0; qq < kNumBasis / 2; ++qq) {
              const float4 v = __ldg(basis4 + k * (kNumBasis / 2) + qq);
              ff_mac(s_hi, s_lo, ch[2 * qq], cl[2 * qq], v.x, v.y);
              ff_mac(s_hi, s_lo, ch[2 * qq + 1], cl[2 * qq + 1], v.z, v.w);
            }
            const float base = __fadd_rn(__fsub_rn(s_hi, rintf(s_hi)), s_lo);
            float zr = 0.f, zi = 0.f;
#pragma unroll
            for (int d = 0; d < D; ++d) {
              const uint32_t top = (uint32_t)k * xh[d] + __umulhi((uint32_t)k, xl[d]);
              float ph = base + __int2float_rn((int)top) * 2.3283064365386963e-10f;
              ph -= rintf(ph);
              float sn, cs;
              __sincosf(ph * 6.283185307179586f, &sn, &cs);
              const float2 w = __ldg(a.w[d] + k);
              const float er = w.x * cs - w.y * sn, ei = w.x * sn + w.y * cs;
              // h conj(d) / S = G conj(e^{i Phi} w)
              zr += gre[d] * er + gim[d] * ei;
              zi += gim[d] * er - gre[d] * ei;
            }
            z2 += zr * zr + zi * zi;
            // Y[v] += z exp(-2 pi i j v / 16)
#pragma unroll
            for (int v = 0; v < 16; ++v) {
              const float2 t = s_w16[(j * v) & 15];
              yr[v] += zr * t.x - zi * t.y;
              yi[v] += zr * t.y + zi * t.x;
            }
          }
#pragma unroll
          for (int v = 0; v < 16; ++v) buf[P(16 * bb + v)] = make_float2(yr[v], yi[v]);
        }
      }
      for (int64_t k = threadIdx.x; a.model != GWL_MODEL_TAYLORF2 && k < L; k += blockDim.x) {
        float zr = 0.f, zi = 0.f;
        const bool in_hull = k >= a.k_lo && k < a.k_hi;
        if (r.valid && in_hull) {
          if (a.model == GWL_MODEL_TAYLORF2) {
            if (k >= r.k_start && k < r.k_end) {
              const float4* bp = reinterpret_cast<const float4*>(a.basis + k * kNumBasis);
              float s_hi = ch[kNumBasis], s_lo = cl[kNumBasis];
#pragma unroll
              for (int q = 0; q < kNumBasis / 2; ++q) {
                const float4 v = bp[q];
                ff_mac(s_hi, s_lo, ch[2 * q], cl[2 * q], v.x, v.y);
                ff_mac(s_hi, s_lo, ch[2 * q + 1], cl[2 * q + 1], v.z, v.w);
              }
              const float base = __fadd_rn(__fsub_rn(s_hi, rintf(s_hi)), s_lo);
#pragma unroll
              for (int d = 0; d < D; ++d) {
                const uint32_t top = (uint32_t)k * xh[d] + __umulhi((uint32_t)k, xl[d]);
                float ph = base + __int2float_rn((int)top) * 2.3283064365386963e-10f;
                ph -= rintf(ph);
                float sn, cs;
                __sincosf(ph * 6.283185307179586f, &sn, &cs);
                const float2 w = a.w[d][k];
                const float er = w.x * cs - w.y * sn, ei = w.x * sn + w.y * cs;
                // h conj(d) / S = G conj(e^{i Phi} w)
                zr += gre[d] * er + gim[d] * ei;
                zi += gim[d] * er - gre[d] * ei;
              }
            }
          } else {
            const float f = a.freq_f[k];
            const float g1 = gauss_ff(f, f0h, f0l, gah, gal, -1.0f);
            const float g2 = gauss_ff(f, f0h, f0l, gah, gal, 1.0f);
            const float hp = g1 + g2, hx = g1 - g2;
#pragma unroll
            for (int d = 0; d < D; ++d) {
              const uint32_t top = (uint32_t)k * xh[d] + __umulhi((uint32_t)k, xl[d]);
              const float ph = __int2float_rn((int)top) * 2.3283064365386963e-10f;
              float sn, cs;
              sincospif(2.0f * ph, &sn, &cs);  // linear phase: avoid coherent approximation error
              const float2 w = a.w[d][k];
              const float er = w.x * cs - w.y * sn, ei = w.x * sn + w.y * cs;
              // (C hp - i E hx) conj(e)
              const float ar = cre[d] * hp, ai = -cim[d] * hx;
              zr += ar * er + ai * ei;
              zi += ai * er - ar * ei;
            }
          }
        }
        buf[P(brpos(k))] = make_float2(zr, zi);
      }
      if (a.model == GWL_MODEL_SINEGAUSSIAN && threadIdx.x == 0 && r.valid) {
        // the float-float <h|h> of the k_mixed_sg pass launched before this
        // kernel (partial sum 2 of every chunk group, in group order)
        const int64_t gs = (int64_t)a.n_det * kPartStride * a.B;
        for (int d = 0; d < D; ++d) {
          const double A = r.fp[d] * r.amp, Cx = r.fx[d] * r.amp2;
          const double* q = a.part + ((int64_t)d * kPartStride + 2) * a.B + i;
          double p2 = 0.0;
          for (int64_t g = 0; g < a.n_chunks; ++g) p2 += q[g * gs];
          hh_part += norm * a.v_scale[d] * (A * A + Cx * Cx) * p2;
        }
      }
    } else if (a.relbin) {
      // relative binning (relative.py:365-396, 398-420): the ratios
      // h_d(f_e) / h0_d(f_e) at the bin edges in shared memory, <h|h> from the
      // summary data, and the integrand from the full-grid waveform
      // h0_d(f) (r0_b + r1_b (f - f_b)) of each bin b
      double2* s_rat = reinterpret_cast<double2*>(smem);  // [D][nE]
      const int nE = a.rb_edges;
      relbin_edge_ratios<D>(a, r, s_rat);
      __syncthreads();
      hh_part = relbin_hh_part<D>(a, s_rat);
      const int64_t k0 = a.rb_index[0], k1 = a.rb_index[nE - 1];
      for (int64_t k = threadIdx.x; k < L; k += blockDim.x) {
        double zr = 0.0, zi = 0.0;
        if (r.valid && k >= k0 && k <= k1) {
          const int b = a.rb_bin[k - k0];
          if (!GWL_INDEX_OK(b, nE - 1, a.status)) continue;
          const double fb0 = a.rb_freq[b], fb1 = a.rb_freq[b + 1];
          const double x = a.freq[k] - (fb1 + fb0) / 2, width = fb1 - fb0;
#pragma unroll
          for (int d = 0; d < D; ++d) {
            const double2 q0 = s_rat[d * nE + b], q1 = s_rat[d * nE + b + 1];
            const double rr = (q1.x + q0.x) / 2 + (q1.x - q0.x) / width * x;
            const double ri = (q1.y + q0.y) / 2 + (q1.y - q0.y) / width * x;
            const double2 g = a.rb_g[d][k];  // 4/T h0 conj(d) / S
            zr += g.x * rr - g.y * ri;
            zi += g.x * ri + g.y * rr;
          }
        }
        buf[brpos(k)] = make_double2(zr, zi);
      }
    } else if (a.mb_tm) {
      // multi-banding (multiband.py:714-726, 792-800): the banded strain
      // times the linear coefficients, scattered to the full-resolution
      // indices int(f_j T) in band order, then the FFT; <h|h> from the
      // quadratic coefficients over every banded point
      const bool tf2 = a.model == GWL_MODEL_TAYLORF2;
      const double u = tf2 ? cbrt(kPi * r.m_sec) : 0.0, lnu = tf2 ? log(u) : 0.0;
      const double pu5 = tf2 ? 3.0 / (128.0 * r.eta) / (u * u * u * u * u) : 0.0;
      for (int64_t k = threadIdx.x; k < L; k += blockDim.x) {
        double zr = 0.0, zi = 0.0;
        const int32_t c1 = a.mb_tm_ptr[k + 1];
        for (int32_t c = a.mb_tm_ptr[k]; r.valid && c < c1; ++c) {
          const int32_t code = a.mb_tm_src[c];
          const int64_t j = code >= 0 ? (int64_t)code : -(int64_t)code - 1;
          if (!GWL_INDEX_OK(j, a.mb_points, a.status)) continue;
          const double f = a.mb_freq[j];
          double2 hp = make_double2(0.0, 0.0), hx = make_double2(0.0, 0.0);
          if (!(tf2 ? tf2_pols_t(a, r, a.mb_pow[j], f, u, lnu, pu5, hp, hx) : plain_pols(a, r, f, hp, hx)))
            continue;
#pragma unroll
          for (int d = 0; d < D; ++d) {
            // interferometer.py:341-362 at explicit frequencies (no mask)
            const double sre = hp.x * r.fp[d] + hx.x * r.fx[d], sim = hp.y * r.fp[d] + hx.y * r.fx[d];
            double sn, cs;
            sincos(2.0 * kPi * r.dt[d] * f, &sn, &cs);
            const double hre = sre * cs + sim * sn, him = sim * cs - sre * sn;
            hh_part += (hre * hre + him * him) * a.mb_quad[d][j];
            if (code >= 0) {
              const double2 w = a.mb_lin[d][j];
              zr += hre * w.x - him * w.y;
              zi += hre * w.y + him * w.x;
            }
          }
        }
        buf[brpos(k)] = make_double2(zr, zi);
      }
    } else {
      // e^{i w f_k} for this thread's bins k = tid, tid + T, ... by rotation
      double zc[D], zs[D], rc[D], rs[D];
      for (int d = 0; d < D; ++d) {
        const double w2 = 2.0 * kPi * r.dt[d];
        sincos(w2 * ((double)threadIdx.x * a.step), &zs[d], &zc[d]);
        sincos(w2 * ((double)blockDim.x * a.step), &rs[d], &rc[d]);
      }
      const bool tf2 = a.model == GWL_MODEL_TAYLORF2;
      const double u = tf2 ? cbrt(kPi * r.m_sec) : 0.0, lnu = tf2 ? log(u) : 0.0;
      const double pu5 = tf2 ? 3.0 / (128.0 * r.eta) / (u * u * u * u * u) : 0.0;
      for (int64_t k = threadIdx.x; k < L; k += blockDim.x) {
        double zr = 0.0, zi = 0.0;
        double2 hp, hx;
        if (r.valid && k >= a.k_lo && k < a.k_hi) {
          const double f = a.freq[k];
          if (tf2 ? tf2_pols_tab(a, r, k, f, u, lnu, pu5, hp, hx) : plain_pols(a, r, f, hp, hx)) {
#pragma unroll
            for (int d = 0; d < D; ++d) {
              const double is = a.inv_psd[d][k];
              if (is == 0.0) continue;
              const double sre = hp.x * r.fp[d] + hx.x * r.fx[d];
              const double sim = hp.y * r.fp[d] + hx.y * r.fx[d];
              const double sn = zs[d], cs = zc[d];
              const double hre = sre * cs + sim * sn, him = sim * cs - sre * sn;
              const double2 dd = reinterpret_cast<const double2*>(a.strain[d])[k];
              // base.py:326-329: signal * conj(d) / S
              zr += (hre * dd.x + him * dd.y) * is;
              zi += (him * dd.x - hre * dd.y) * is;
              hh_part += (hre * hre + him * him) * is;
            }
          }
        }
        buf[brpos(k)] = make_double2(norm * zr, norm * zi);
#pragma unroll
        for (int d = 0; d < D; ++d) tm_rotate(zc[d], zs[d], rc[d], rs[d]);
      }
      hh_part *= norm;
    }
    // The last bin (index L) only enters <h|h>; the FFT uses bins 0..L-1.
    if (!MIXED && !a.relbin && !a.mb_tm && threadIdx.x == 0 && r.valid && L >= a.k_lo && L < a.k_hi) {
      double2 hp, hx;
      const double f = a.freq[L];
      if (plain_pols(a, r, f, hp, hx)) {
        for (int d = 0; d < D; ++d) {
          const double is = a.inv_psd[d][L];
          const double sre = hp.x * r.fp[d] + hx.x * r.fx[d], sim = hp.y * r.fp[d] + hx.y * r.fx[d];
          hh_part += norm * (sre * sre + sim * sim) * is;
        }
      }
    }
    if (MIXED && threadIdx.x == 0) {
      // this point's window of FFT indices inside the prior (exact, from the
      // prologue): the last FFT stages compute only the outputs inside it
      s_jr[0] = r.tm_j0;
      s_jr[1] = r.tm_j1;
    }
    __syncthreads();
    // ---- B: in-place FFT, radix-4 passes (two radix-2 stages each) -------
    const int64_t n_win = MIXED ? (int64_t)(s_jr[1] - s_jr[0] + 1) : 0;
    int stage = 1;
    if (MIXED && a.model == GWL_MODEL_TAYLORF2) {
      stage = 5;  // stages 1-4 ran with the integrand
    } else if (log2N & 1) {  // one radix-2 stage first when log2 N is odd
      for (int64_t bf = threadIdx.x; bf < L / 2; bf += blockDim.x) {
        const int64_t i0 = 2 * bf, i1 = i0 + 1;
        const C x0 = buf[P(i0)], x1 = buf[P(i1)];
        C y0, y1;
        y0.x = x0.x + x1.x;
        y0.y = x0.y + x1.y;
        y1.x = x0.x - x1.x;
        y1.y = x0.y - x1.y;
        buf[P(i0)] = y0;
        buf[P(i1)] = y1;
      }
      __syncthreads();
      stage = 2;
    }
    {
      // radix-16 passes (mixed; radix-8 in float64, within the register
      // budget): RB radix-2 stages in registers, fewer round trips through the
      // buffer and fewer barriers; the stage-j twiddles of a group depend only
      // on (k mod 2^j)
      constexpr int RB = MIXED ? 4 : 3, RN = 1 << RB;
      for (; stage + RB - 1 <= log2N; stage += RB) {
        const int64_t h0 = (int64_t)1 << (stage - 1);
        for (int64_t gi = threadIdx.x; gi < L / RN; gi += blockDim.x) {
          const int64_t pos = gi & (h0 - 1);
          const int64_t b0 = ((gi >> (stage - 1)) << (stage - 1 + RB)) + pos;
          C x[RN];
#pragma unroll
          for (int k = 0; k < RN; ++k) x[k] = buf[P(b0 + k * h0)];
#pragma unroll
          for (int j = 0; j < RB; ++j) {
            // exp(-2 pi i (pos + m h0) L / (2 h0 2^j) / L) = tw(pos stride) * exp(-2 pi i m / 2^(j+1))
            const int64_t stride = L >> (stage + j);  // L / (2 h0 2^j), L = m_odd 2^log2N
            C w[MIXED ? 8 : 1];
            if constexpr (MIXED) {
              const C w0 = tw(pos * stride);
              w[0] = w0;
#pragma unroll
              for (int m = 1; m < (1 << j); ++m) {
                const float2 u = s_w16[m << (3 - j)];
                w[m].x = w0.x * u.x - w0.y * u.y;
                w[m].y = w0.x * u.y + w0.y * u.x;
              }
            }
#pragma unroll
            for (int k = 0; k < RN; ++k) {
              if (k & (1 << j)) continue;
              const int k2 = k | (1 << j);
              // float64: each twiddle from the table (few registers),
              // exp(-2 pi i (pos + m h0) stride / L) for m = k mod 2^j
              C ww;
              if constexpr (MIXED) ww = w[k & ((1 << j) - 1)];
              else ww = tw((pos + (int64_t)(k & ((1 << j) - 1)) * h0) * stride);
              const R tr = ww.x * x[k2].x - ww.y * x[k2].y, ti = ww.x * x[k2].y + ww.y * x[k2].x;
              x[k2].x = x[k].x - tr;
              x[k2].y = x[k].y - ti;
              x[k].x = x[k].x + tr;
              x[k].y = x[k].y + ti;
            }
          }
#pragma unroll
          for (int k = 0; k < RN; ++k) buf[P(b0 + k * h0)] = x[k];
        }
        __syncthreads();
      }
    }
    for (; stage < log2N; stage += 2) {
      const int64_t h = (int64_t)1 << (stage - 1);  // half-length of the first of the two stages
      const int64_t s1 = L / (2 * h), s2 = L / (4 * h);  // twiddle strides of the two stages
      // mixed, the last two stages (h = N / 4): output j of each block comes
      // from the block's butterfly at j mod h alone, so only the window's run
      const bool prune = MIXED && stage + 1 == log2N && n_win > 0 && n_win <= h;
      const int64_t n_bf = prune ? n_win * m_odd : L / 4;
      for (int64_t t = threadIdx.x; t < n_bf; t += blockDim.x) {
        // pruned: butterfly (s_jr[0] + t mod n_win) mod h of transform t / n_win (32-bit division, none for m_odd = 1)
        const uint32_t tq = (prune && m_odd != 1) ? (uint32_t)t / (uint32_t)n_win : 0u;
        const int64_t tr_ = prune ? (int64_t)((uint32_t)t - tq * (uint32_t)n_win) : 0;
        const int64_t bf = prune ? ((int64_t)tq * h + ((s_jr[0] + tr_) & (h - 1))) : t;
        const int64_t pos = bf & (h - 1);
        const int64_t i0 = ((bf >> (stage - 1)) << (stage + 1)) + pos;
        const int64_t i1 = i0 + h, i2 = i0 + 2 * h, i3 = i0 + 3 * h;
        const C w1 = tw(pos * s1), w2 = tw(pos * s2), w3 = tw((pos + h) * s2);
        const C x0 = buf[P(i0)], x1 = buf[P(i1)], x2 = buf[P(i2)], x3 = buf[P(i3)];
        C a0, a1, a2, a3, y0, y1, y2, y3;
        R tr = w1.x * x1.x - w1.y * x1.y, ti = w1.x * x1.y + w1.y * x1.x;
        a0.x = x0.x + tr; a0.y = x0.y + ti; a1.x = x0.x - tr; a1.y = x0.y - ti;
        tr = w1.x * x3.x - w1.y * x3.y; ti = w1.x * x3.y + w1.y * x3.x;
        a2.x = x2.x + tr; a2.y = x2.y + ti; a3.x = x2.x - tr; a3.y = x2.y - ti;
        tr = w2.x * a2.x - w2.y * a2.y; ti = w2.x * a2.y + w2.y * a2.x;
        y0.x = a0.x + tr; y0.y = a0.y + ti; y2.x = a0.x - tr; y2.y = a0.y - ti;
        tr = w3.x * a3.x - w3.y * a3.y; ti = w3.x * a3.y + w3.y * a3.x;
        y1.x = a1.x + tr; y1.y = a1.y + ti; y3.x = a1.x - tr; y3.y = a1.y - ti;
        buf[P(i0)] = y0;
        buf[P(i1)] = y1;
        buf[P(i2)] = y2;
        buf[P(i3)] = y3;
      }
      __syncthreads();
    }
    if (stage == log2N) {  // a last radix-2 stage (half-length N / 2, twiddle exp(-2 pi i l / N))
      const int64_t h = N2 / 2;
      const bool prune = MIXED && n_win > 0 && n_win <= h;  // only the window's butterflies
      const int64_t n_bf = prune ? n_win * m_odd : L / 2;
      for (int64_t t = threadIdx.x; t < n_bf; t += blockDim.x) {
        // t / n_win (pruned, 32-bit; none for m_odd = 1) or t / h (h = 2^(log2N - 1))
        const uint32_t tq = prune ? (m_odd == 1 ? 0u : (uint32_t)t / (uint32_t)n_win) : (uint32_t)(t >> (log2N - 1));
        // (prune implies n_win > 0)
        const int64_t l = prune ? ((s_jr[0] + (int64_t)((uint32_t)t - tq * (uint32_t)n_win)) & (h - 1)) : (t & (h - 1));
        const int64_t q = (int64_t)tq * N2 + l;
        const C w = tw(l * m_odd);
        const C x0 = buf[P(q)], x1 = buf[P(q + h)];
        const R tr = w.x * x1.x - w.y * x1.y, ti = w.x * x1.y + w.y * x1.x;
        C y0, y1;
        y0.x = x0.x + tr;
        y0.y = x0.y + ti;
        y1.x = x0.x - tr;
        y1.y = x0.y - ti;
        buf[P(q)] = y0;
        buf[P(q + h)] = y1;
      }
      __syncthreads();
    }
    // ---- C: prior window, marginalised lnL per time sample, logsumexp ----
    double hh = 0.0;
    if (!(MIXED && a.model == GWL_MODEL_TAYLORF2)) hh = block_sum(hh_part, red);
    if constexpr (!MIXED) {
      if (a.tm_series) {
        // the whole transform in natural order, d_inner_h_array of
        // base.py:325-330, and <h|h> (block_sum ends with a barrier, so the
        // last FFT stage's writes are visible)
        double2* dst = reinterpret_cast<double2*>(a.tm_series) + (size_t)i * L;
        for (int64_t k = threadIdx.x; k < L; k += blockDim.x) dst[k] = out_at(buf, k);
        if (a.hh_out && threadIdx.x == 0) a.hh_out[i] = hh;
      }
    }
    const double jit = r.jitter;
    // per-point scalars: the TaylorF2 <h|h> from the prologue
    if (MIXED && a.model == GWL_MODEL_TAYLORF2) hh = r.tm_hh;
    if (MIXED && (threadIdx.x == 0 || threadIdx.x == 32)) {
      // the divisions precomputed on the host (LaunchArgs::tm_step ...);
      // thread 0 the scalars, thread 32 (another warp) the distance spline's
      // row at this point's <h|h>, at the same time
      const double sr = r.dist * a.inv_ref_dist;
      const double hh_ref = hh * sr * sr;
      if (threadIdx.x == 0) {
        s_scal[0] = hh;
        s_scal[1] = hh_ref;
        s_scal[2] = sr;
        s_scal[3] = a.tm_step;
        s_scal[4] = a.tm_prob;
        // the window (s_jr) was set before the FFT
      } else if (a.dist_marg) {
        if (a.model == GWL_MODEL_TAYLORF2) {  // computed by the prologue
          s_row.Ly = r.tm_row_ly;
          s_row.inside = r.tm_row_in;
          for (int q = 0; q < 4; ++q) s_row.hy[q] = r.tm_row_hy[q];
        } else {
          s_row = bicubic_row_f(s_ty, a.ny, a.bbox, (float)hh_ref);
        }
      }
    }
    if (!MIXED && threadIdx.x == 0) {
      const double step = a.duration / (double)L;  // linspace(0, T, L + 1) spacing
      s_scal[3] = step;
      s_scal[4] = 1.0 / (a.t_max - a.t_min);
      s_scal[0] = hh;
      s_scal[1] = hh * r.dist * r.dist / (a.ref_dist * a.ref_dist);
      s_scal[2] = r.dist / a.ref_dist;
      // candidate window from the real-valued bounds, checked exactly below
      const double jl = floor((a.t_min - a.start_time0 - jit) / step) - 3.0;
      const double jh = ceil((a.t_max - a.start_time0 - jit) / step) + 2.0;
      s_jr[0] = (long long)fmax(0.0, jl);
      s_jr[1] = (long long)fmin((double)(L - 1), jh);
    }
    __syncthreads();
    hh = s_scal[0];
    const double hh_ref = s_scal[1], sr = s_scal[2], step = s_scal[3], prob = s_scal[4];
    const int64_t j_lo = s_jr[0], j_hi = s_jr[1];
    // one pass: running (max, sum of exp(l - max)) per thread, then a fixed-order block combination
    double m = -INFINITY, acc = 0.0;
    float xmax = 0.f;  // mixed: the largest |X| over this thread's samples (error bound)
    float mf32 = -INFINITY, acc32 = 0.f;  // mixed: the same in float32, without the point's constant -<h|h>/2
    if constexpr (MIXED) {
      // every sample of [j_lo, j_hi] is inside the prior; the per-sample lnL
      // without the constant term (-<h|h>/2 unless the distance table holds
      // it), in float32 throughout
      const float srf = (float)sr;
      for (int64_t j = j_lo + threadIdx.x; j <= j_hi; j += blockDim.x) {
        float lw = 0.f;
        if (a.tm_prior) {
          const float pw = tm_prior_density_f(a, tm_sample_time(a, j, L, step, jit));  // base.py:807, prior(t_j)
          if (!(pw > 0.f)) continue;
          lw = __logf(pw);
        }
        const C x = out_at(buf, j);
        const float ax = sqrtf(x.x * x.x + x.y * x.y);
        float l;
        if (a.dist_marg) {
          l = bicubic_eval_row_ff(s_tx, a.nx, a.ny, a.tc_f, a.bbox_x_f, (a.phase_marg ? ax : x.x) * srf, s_row);
        } else if (a.phase_marg) {
          l = ax + ln_i0_minus_x(ax);
        } else {
          l = x.x;
        }
        l += lw;
        xmax = fmaxf(xmax, ax);
        if (l > mf32) {
          acc32 = mf32 > -INFINITY ? acc32 * __expf(mf32 - l) + 1.f : 1.f;
          mf32 = l;
        } else if (isfinite(l)) {
          acc32 += __expf(l - mf32);
        }
      }
    } else {
      for (int64_t j = j_lo + threadIdx.x; j <= j_hi; j += blockDim.x) {
        const double t = tm_sample_time(a, j, L, step, jit);
        double lw;
        if (!tm_log_weight<MIXED>(a, t, lw)) continue;
        const C x = out_at(buf, j);
        const double l = tm_lnl_fp64(a, x.x, x.y, hh, hh_ref, sr);
        tm_lse_push<MIXED>(l + lw, m, acc);
      }
    }
    // combine (m, acc) pairs over the block in a fixed order
    double* redm = red;
    double* reds = red + kTmThreads;
    if constexpr (MIXED) {
      // all warps: the maximum of the threads' m as float32 (any reference
      // near the maximum serves), then sum acc_t exp(m_t - M) in float32; both
      // by xor-shuffles within warps and a fixed-order sum of the 16 warps
      const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
      float mf = mf32, zz = z2, xm = xmax;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        mf = fmaxf(mf, __shfl_xor_sync(0xffffffffu, mf, o));
        zz += __shfl_xor_sync(0xffffffffu, zz, o);
        xm = fmaxf(xm, __shfl_xor_sync(0xffffffffu, xm, o));
      }
      float* redf = reinterpret_cast<float*>(reds);
      if (lane == 0) {
        redf[warp] = mf;
        redf[kTmThreads / 32 + warp] = zz;       // error bound: sum of |z|^2 ...
        redf[2 * (kTmThreads / 32) + warp] = xm;  // ... and the largest |X|
      }
      __syncthreads();
      float M = redf[0];
      for (int w = 1; w < kTmThreads / 32; ++w) M = fmaxf(M, redf[w]);
      float sm = 0.f;
      if (isfinite(M) && isfinite(mf32)) sm = acc32 * __expf(mf32 - M);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) sm += __shfl_xor_sync(0xffffffffu, sm, o);
      __syncthreads();
      if (lane == 0) redf[warp] = sm;
      __syncthreads();
      if (threadIdx.x == 0) {
        float total = 0.f, zs = 0.f, xp = 0.f;
        for (int w = 0; w < kTmThreads / 32; ++w) {
          total += redf[w];
          zs += redf[kTmThreads / 32 + w];
          xp = fmaxf(xp, redf[2 * (kTmThreads / 32) + w]);
        }
        redm[0] = isfinite(M) ? (double)M : -INFINITY;
        redm[1] = sqrt((double)zs);
        redm[2] = (double)xp;
        reds[0] = (double)total;
      }
      __syncthreads();
    } else {
      redm[threadIdx.x] = m;
      reds[threadIdx.x] = acc;
      __syncthreads();
      for (int w = kTmThreads / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) {
          const double m1 = redm[threadIdx.x], m2 = redm[threadIdx.x + w];
          const double s1 = reds[threadIdx.x], s2 = reds[threadIdx.x + w];
          const double mm = fmax(m1, m2);
          double ss = 0.0;
          if (isfinite(mm)) ss = (isfinite(m1) ? s1 * exp(m1 - mm) : 0.0) + (isfinite(m2) ? s2 * exp(m2 - mm) : 0.0);
          redm[threadIdx.x] = mm;
          reds[threadIdx.x] = ss;
        }
        __syncthreads();
      }
    }
    if (threadIdx.x == 0) {
      // mixed: the maximum is of the per-sample lnL without the point's
      // constant, added here in float64
      const double c0 = MIXED && !a.dist_marg ? -hh / 2 : 0.0;
      const double amax = redm[0] + c0, total = reds[0] * (a.tm_prior ? 1.0 : prob) * a.delta_tc;
      double lnl;
      if (!r.valid) lnl = -1.7976931348623157e308;
      else if (!isfinite(amax)) lnl = amax;
      // mixed: the logarithm of the O(1..1e3) sum in float32 (error ~1e-7)
      else lnl = amax + (MIXED ? (double)logf((float)total) : log(total));
      a.out[i] = lnl;
      if (MIXED && a.model == GWL_MODEL_TAYLORF2 && a.rf_tol > 0 && a.rf_count && a.rf_list && r.valid) {
        // the error bound's inputs, for k_tm_marks (so that no thread of this
        // CTA holds the others up with the distance table's sensitivity)
        a.rec[i].tm_xp = (float)redm[2];
        a.rec[i].tm_zs = (float)redm[1];
      }
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// Mixed TaylorF2 time marginalisation in two half-length transforms.  With
// L = 2 M (M a power of two, at least 32), X[j] = E[j mod M] +
// e^{-2 pi i j / L} O[j mod M], E and O the length-M transforms of the even
// and the odd bins (the last radix-2 stage of a decimation in time).  One CTA
// of 256 threads per point runs E, keeps its values at the prior window's
// samples, then O in the same shared buffer, and combines them there: the
// buffer is half of k_time_marg's, so two CTAs (two points, each in its own
// phase of the work) share an SM.  Each half runs as k_time_marg<D, true>
// runs its transform: the integrand fused with the first four stages, radix-16
// passes in registers, the last passes only for the window's outputs; then
// the window in float32 and the error bound's inputs, as there.
// ---------------------------------------------------------------------------
// LS = 1 splits the transform in two (256 threads per CTA, two CTAs per SM),
// LS = 2 in four (X[j] = sum_r e^{-2 pi i j r / L} Y_r[j mod L/4], Y_r over the
// bins k = 4 k' + r; 128 threads, four CTAs per SM).
constexpr int kTmHalfLs = 2;

template <int D, int LS>
__global__ void __launch_bounds__(512 >> LS, 1 << LS) k_tm_half(LaunchArgs a, const float2* twiddle, int log2L,
                                                                  int n_win_cap) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ float s_coef[2 * kMaxDet];
  __shared__ SplineRowF s_row;
  __shared__ float2 tw_hi[kTmTwiddleRows], tw_lo[kTmTwiddleRows];
  __shared__ float2 s_w16[16];
  constexpr int W = (512 >> LS) / 32;
  __shared__ float redf[4 * W];
  const int64_t L = a.n_fft, M = L >> LS;
  const int lM = log2L - LS;
  const int64_t hL = L >> 1;  // the table holds exp(-2 pi i q / L) for q < L / 2
  for (int q = threadIdx.x; q < kTmTwiddleRows; q += blockDim.x) {
    const int64_t qh = (int64_t)q * kTmTwiddleRows;
    tw_hi[q] = qh < hL ? twiddle[qh] : make_float2(1.f, 0.f);
    tw_lo[q] = q < hL ? twiddle[q] : make_float2(1.f, 0.f);
  }
  if (threadIdx.x < 8) {  // the 16th roots of unity exp(-2 pi i m / 16)
    const float2 t = twiddle[(int64_t)threadIdx.x * (L / 16)];
    s_w16[threadIdx.x] = t;
    s_w16[threadIdx.x + 8] = make_float2(-t.x, -t.y);
  }
  float2* buf = reinterpret_cast<float2*>(smem);  // [M + M / 16], padded every 16
  float2* s_ew = buf + (M + (M >> 4));            // [n_win_cap] the window's values
  float* s_tx = reinterpret_cast<float*>(s_ew + n_win_cap);
  float* s_ty = s_tx + a.nx;
  if (a.dist_marg) {
    for (int q = threadIdx.x; q < a.nx; q += blockDim.x) s_tx[q] = a.tx_f[q];
    for (int q = threadIdx.x; q < a.ny; q += blockDim.x) s_ty[q] = a.ty_f[q];
  }
  __syncthreads();
  // exp(-2 pi i q / L), q < L / 2, from the two tables
  const auto tw = [&](int64_t q) -> float2 {
    const float2 h = tw_hi[q / kTmTwiddleRows], l = tw_lo[q % kTmTwiddleRows];
    return make_float2(h.x * l.x - h.y * l.y, h.x * l.y + h.y * l.x);
  };
  const auto P = [](int64_t q) -> int64_t { return q + (q >> 4); };
  const float4* basis4 = reinterpret_cast<const float4*>(a.basis);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int64_t i = blockIdx.x; i < a.B; i += gridDim.x) {
    const PointRec& r = a.rec[i];
    if (threadIdx.x < 2 * D) s_coef[threadIdx.x] = r.tm_coef[threadIdx.x];
    const int64_t j_lo = r.tm_j0;
    int64_t n_win = r.tm_j1 - r.tm_j0 + 1;
    if (n_win > n_win_cap) {  // cannot happen: the host sizes the window from the prior's width
      if (threadIdx.x == 0 && a.status) atomicExch(a.status, kDevStatusBadInput);
      n_win = n_win_cap;
    }
    __syncthreads();
    float gre[D], gim[D];
    uint32_t xl[D], xh[D];
    float ch[kNumBasis + 1], cl[kNumBasis + 1];
#pragma unroll
    for (int d = 0; d < D; ++d) {
      xl[d] = r.xfix[d][0];
      xh[d] = r.xfix[d][1];
      gre[d] = s_coef[2 * d];
      gim[d] = s_coef[2 * d + 1];
    }
#pragma unroll
    for (int b = 0; b <= kNumBasis; ++b) {
      ch[b] = r.c_hi[b];
      cl[b] = r.c_lo[b];
    }
    const int64_t ks = max(r.k_start, a.k_lo), ke = min(min(r.k_end, a.k_hi), L);
    float z2 = 0.f;  // sum of |z_k|^2 over this thread's bins (error bound)
    for (int par = 0; par < (1 << LS); ++par) {
      // ---- A: bins k = 2^LS k' + par, fused with the first four stages: after
      // them positions 16 b .. 16 b + 15 hold the 16-point DFT of the bins
      // k' = q + j M / 16 (j < 16), q = bitrev(b) over log2(M) - 4 bits
      const int64_t R = M >> 4;
      const int lr = lM - 4;
      // in-band k' in [ka, kb)
      const int64_t ka = (ks - par + (1 << LS) - 1) >> LS, kb = (ke - par + (1 << LS) - 1) >> LS;
      for (int64_t bb = threadIdx.x; bb < R; bb += blockDim.x) {
        const int64_t q = (int64_t)bit_reverse((uint32_t)bb, lr);
        float yr[16], yi[16];
#pragma unroll
        for (int v = 0; v < 16; ++v) yr[v] = yi[v] = 0.f;
        const int j0 = r.valid ? (ka > q ? (int)(((uint32_t)(ka - q) + (uint32_t)R - 1u) >> lr) : 0) : 16;
        const int j1 = r.valid ? (kb > q ? min(16, (int)(((uint32_t)(kb - q) + (uint32_t)R - 1u) >> lr)) : 0) : 0;
        for (int j = j0; j < j1; ++j) {
          const int64_t k = ((q + (int64_t)j * R) << LS) + par;
          float s_hi = ch[kNumBasis], s_lo = cl[kNumBasis];
#pragma unroll
          for (int qq = 0; qq < kNumBasis / 2; ++qq) {
            const float4 v = __ldg(basis4 + k * (kNumBasis / 2) + qq);
            ff_mac(s_hi, s_lo, ch[2 * qq], cl[2 * qq], v.x, v.y);
            ff_mac(s_hi, s_lo, ch[2 * qq + 1], cl[2 * qq + 1], v.z, v.w);
          }
          const float base = __fadd_rn(__fsub_rn(s_hi, rintf(s_hi)), s_lo);
          float zr = 0.f, zi = 0.f;
#pragma unroll
          for (int d = 0; d < D; ++d) {
            const uint32_t top = (uint32_t)k * xh[d] + __umulhi((uint32_t)k, xl[d]);
            float ph = base + __int2float_rn((int)top) * 2.3283064365386963e-10f;
            ph -= rintf(ph);
            float sn, cs;
            __sincosf(ph * 6.283185307179586f, &sn, &cs);
            const float2 w = __ldg(a.w[d] + k);
            const float er = w.x * cs - w.y * sn, ei = w.x * sn + w.y * cs;
            // h conj(d) / S = G conj(e^{i Phi} w)
            zr += gre[d] * er + gim[d] * ei;
            zi += gim[d] * er - gre[d] * ei;
          }
          z2 += zr * zr + zi * zi;
#pragma unroll
          for (int v = 0; v < 16; ++v) {
            const float2 t = s_w16[(j * v) & 15];
            yr[v] += zr * t.x - zi * t.y;
            yi[v] += zr * t.y + zi * t.x;
          }
        }
#pragma unroll
        for (int v = 0; v < 16; ++v) buf[P(16 * bb + v)] = make_float2(yr[v], yi[v]);
      }
      __syncthreads();
      // ---- B: stages 5 .. log2(M); a stage of half-length h has twiddles
      // exp(-2 pi i pos / (2 h)) = tw(pos L / (2 h))
      int stage = 5;
      for (; stage + 3 <= lM; stage += 4) {
        const int64_t h0 = (int64_t)1 << (stage - 1);
        for (int64_t gi = threadIdx.x; gi < (M >> 4); gi += blockDim.x) {
          const int64_t pos = gi & (h0 - 1);
          const int64_t b0 = ((gi >> (stage - 1)) << (stage + 3)) + pos;
          float2 x[16];
#pragma unroll
          for (int k = 0; k < 16; ++k) x[k] = buf[P(b0 + k * h0)];
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            const float2 w0 = tw(pos * (L >> (stage + j)));
            float2 w[8];
            w[0] = w0;
#pragma unroll
            for (int m = 1; m < (1 << j); ++m) {
              const float2 u = s_w16[m << (3 - j)];
              w[m] = make_float2(w0.x * u.x - w0.y * u.y, w0.x * u.y + w0.y * u.x);
            }
#pragma unroll
            for (int k = 0; k < 16; ++k) {
              if (k & (1 << j)) continue;
              const int k2 = k | (1 << j);
              const float2 ww = w[k & ((1 << j) - 1)];
              const float tr = ww.x * x[k2].x - ww.y * x[k2].y, ti = ww.x * x[k2].y + ww.y * x[k2].x;
              x[k2].x = x[k].x - tr;
              x[k2].y = x[k].y - ti;
              x[k].x = x[k].x + tr;
              x[k].y = x[k].y + ti;
            }
          }
#pragma unroll
          for (int k = 0; k < 16; ++k) buf[P(b0 + k * h0)] = x[k];
        }
        __syncthreads();
      }
      for (; stage < lM; stage += 2) {
        const int64_t h = (int64_t)1 << (stage - 1);
        const int64_t s1 = L >> stage, s2 = L >> (stage + 1);  // L / (2 h), L / (4 h)
        // the last two stages: output j comes from the butterfly at j mod h alone
        const bool prune = stage + 1 == lM && n_win > 0 && n_win <= h;
        const int64_t n_bf = prune ? n_win : (M >> 2);
        for (int64_t t = threadIdx.x; t < n_bf; t += blockDim.x) {
          const int64_t bf = prune ? ((j_lo + t) & (h - 1)) : t;
          const int64_t pos = bf & (h - 1);
          const int64_t i0 = ((bf >> (stage - 1)) << (stage + 1)) + pos;
          const int64_t i1 = i0 + h, i2 = i0 + 2 * h, i3 = i0 + 3 * h;
          const float2 w1 = tw(pos * s1), w2 = tw(pos * s2), w3 = tw((pos + h) * s2);
          const float2 x0 = buf[P(i0)], x1 = buf[P(i1)], x2 = buf[P(i2)], x3 = buf[P(i3)];
          float2 a0, a1, a2, a3, y0, y1, y2, y3;
          float tr = w1.x * x1.x - w1.y * x1.y, ti = w1.x * x1.y + w1.y * x1.x;
          a0.x = x0.x + tr; a0.y = x0.y + ti; a1.x = x0.x - tr; a1.y = x0.y - ti;
          tr = w1.x * x3.x - w1.y * x3.y; ti = w1.x * x3.y + w1.y * x3.x;
          a2.x = x2.x + tr; a2.y = x2.y + ti; a3.x = x2.x - tr; a3.y = x2.y - ti;
          tr = w2.x * a2.x - w2.y * a2.y; ti = w2.x * a2.y + w2.y * a2.x;
          y0.x = a0.x + tr; y0.y = a0.y + ti; y2.x = a0.x - tr; y2.y = a0.y - ti;
          tr = w3.x * a3.x - w3.y * a3.y; ti = w3.x * a3.y + w3.y * a3.x;
          y1.x = a1.x + tr; y1.y = a1.y + ti; y3.x = a1.x - tr; y3.y = a1.y - ti;
          buf[P(i0)] = y0;
          buf[P(i1)] = y1;
          buf[P(i2)] = y2;
          buf[P(i3)] = y3;
        }
        __syncthreads();
      }
      if (stage == lM) {  // a last radix-2 stage, half-length M / 2, twiddle exp(-2 pi i l / M) = tw(2^LS l)
        const int64_t h = M >> 1;
        const bool prune = n_win > 0 && n_win <= h;
        const int64_t n_bf = prune ? n_win : h;
        for (int64_t t = threadIdx.x; t < n_bf; t += blockDim.x) {
          const int64_t l = prune ? ((j_lo + t) & (h - 1)) : t;
          const float2 w = tw(l << LS);
          const float2 x0 = buf[P(l)], x1 = buf[P(l + h)];
          const float tr = w.x * x1.x - w.y * x1.y, ti = w.x * x1.y + w.y * x1.x;
          buf[P(l)] = make_float2(x0.x + tr, x0.y + ti);
          buf[P(l + h)] = make_float2(x0.x - tr, x0.y - ti);
        }
        __syncthreads();
      }
      // the window's values: X = sum over the parts of exp(-2 pi i j par / L) Y_par
      for (int64_t t = threadIdx.x; t < n_win; t += blockDim.x) {
        const int64_t j = j_lo + t;
        const float2 v = buf[P(j & (M - 1))];
        if (par == 0) {
          s_ew[t] = v;
        } else {
          const int64_t qq = (j * par) & (L - 1);
          float2 w = qq < hL ? tw(qq) : tw(qq - hL);
          if (qq >= hL) w = make_float2(-w.x, -w.y);
          const float2 e = s_ew[t];
          s_ew[t] = make_float2(e.x + (w.x * v.x - w.y * v.y), e.y + (w.x * v.y + w.y * v.x));
        }
      }
      __syncthreads();
    }
    // ---- C: the prior window, per sample in float32 without the point's
    // constant -<h|h>/2 (added once at the end), and a logsumexp
    const double hh = r.tm_hh, sr = r.dist * a.inv_ref_dist;
    if (a.dist_marg && threadIdx.x == 0) {
      s_row.Ly = r.tm_row_ly;
      s_row.inside = r.tm_row_in;
      for (int q = 0; q < 4; ++q) s_row.hy[q] = r.tm_row_hy[q];
    }
    __syncthreads();
    const float srf = (float)sr;
    const double jit = r.jitter, step = a.tm_step;
    float mf32 = -INFINITY, acc32 = 0.f, xmax = 0.f;
    for (int64_t t = threadIdx.x; t < n_win; t += blockDim.x) {
      float lw = 0.f;
      if (a.tm_prior) {
        const float pw = tm_prior_density_f(a, tm_sample_time(a, j_lo + t, L, step, jit));  // base.py:807
        if (!(pw > 0.f)) continue;
        lw = __logf(pw);
      }
      const float2 x = s_ew[t];
      const float ax = sqrtf(x.x * x.x + x.y * x.y);
      float l;
      if (a.dist_marg) {
        l = bicubic_eval_row_ff(s_tx, a.nx, a.ny, a.tc_f, a.bbox_x_f, (a.phase_marg ? ax : x.x) * srf, s_row);
      } else if (a.phase_marg) {
        l = ax + ln_i0_minus_x(ax);
      } else {
        l = x.x;
      }
      l += lw;
      xmax = fmaxf(xmax, ax);
      if (l > mf32) {
        acc32 = mf32 > -INFINITY ? acc32 * __expf(mf32 - l) + 1.f : 1.f;
        mf32 = l;
      } else if (isfinite(l)) {
        acc32 += __expf(l - mf32);
      }
    }
    // the block's logsumexp: the float32 maximum, then sum acc_t exp(m_t - M),
    // xor-shuffles within warps and a fixed-order sum over the warps
    float mf = mf32, zz = z2, xm = xmax;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      mf = fmaxf(mf, __shfl_xor_sync(0xffffffffu, mf, o));
      zz += __shfl_xor_sync(0xffffffffu, zz, o);
      xm = fmaxf(xm, __shfl_xor_sync(0xffffffffu, xm, o));
    }
    if (lane == 0) {
      redf[warp] = mf;
      redf[W + warp] = zz;
      redf[2 * W + warp] = xm;
    }
    __syncthreads();
    float Mx = redf[0];
    for (int w = 1; w < W; ++w) Mx = fmaxf(Mx, redf[w]);
    float sm = 0.f;
    if (isfinite(Mx) && isfinite(mf32)) sm = acc32 * __expf(mf32 - Mx);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) sm += __shfl_xor_sync(0xffffffffu, sm, o);
    if (lane == 0) redf[3 * W + warp] = sm;
    __syncthreads();
    if (threadIdx.x == 0) {
      float total = 0.f, zs = 0.f, xp = 0.f;
      for (int w = 0; w < W; ++w) {
        total += redf[3 * W + w];
        zs += redf[W + w];
        xp = fmaxf(xp, redf[2 * W + w]);
      }
      const double c0 = a.dist_marg ? 0.0 : -hh / 2;
      const double amax = (isfinite(Mx) ? (double)Mx : -INFINITY) + c0;
      const double tot = (double)total * (a.tm_prior ? 1.0 : a.tm_prob) * a.delta_tc;
      double lnl;
      if (!r.valid) lnl = -1.7976931348623157e308;
      else if (!isfinite(amax)) lnl = amax;
      else lnl = amax + (double)logf((float)tot);
      a.out[i] = lnl;
      if (a.rf_tol > 0 && a.rf_count && a.rf_list && r.valid) {
        a.rec[i].tm_xp = xp;
        a.rec[i].tm_zs = sqrtf(zs);
      }
    }
    __syncthreads();
  }
}

// The mixed full-grid kernel's error bounds, one thread per point:
// |dlnL| <= s (kTmErrNorm ||z||_2 + kTmErrPeak max|X|), s the distance table's
// sensitivity at the window's peak (tm_sensitivity); points over the
// tolerance are listed for the float64 recomputation.
__global__ void k_tm_marks(LaunchArgs a) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.B) return;
  const PointRec& r = a.rec[i];
  if (!r.valid) return;
  SplineRowF row;
  row.Ly = r.tm_row_ly;
  row.inside = r.tm_row_in;
  for (int q = 0; q < 4; ++q) row.hy[q] = r.tm_row_hy[q];
  const double xp = (double)r.tm_xp, sr = r.dist * a.inv_ref_dist;
  const double err = tm_sensitivity(a, xp, sr, a.tx_f, row) * (kTmErrNorm * (double)r.tm_zs + kTmErrPeak * xp);
  if (!(err <= a.rf_tol)) {
    a.rec[i].refine = 1;
    a.rf_list[atomicAdd(a.rf_count, 1)] = (int32_t)i;
  }
}

cudaError_t launch_time_marg_marks(const LaunchArgs& a, cudaStream_t s) {
  if (a.precision != GWL_PRECISION_MIXED || a.model != GWL_MODEL_TAYLORF2 || !(a.rf_tol > 0) || !a.rf_count ||
      !a.rf_list || a.B <= 0)
    return cudaSuccess;
  k_tm_marks<<<(unsigned)((a.B + 127) / 128), 128, 0, s>>>(a);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// ROQ with time marginalisation (roq.py:320-331, 467-541, 604-651, with
// base.py:794-820): one CTA per point.
//   1. conj(h_d) at the linear nodes into shared memory (antenna patterns at
//      the prior's mid time, no time shift), <h|h> from the quadratic nodes;
//   then per chunk of roq_tm_chunk time samples:
//   2. D_d[k] = sum_q W_d[k][q] conj(h_d(F_q)) for the weight rows k the
//      chunk's samples read (one warp per row, fixed-order reduction);
//   3. for each time sample t_j of the marginalisation grid inside the prior,
//      <d|h>(t_j) = sum_d of the five-sample interpolation of D_d at the
//      detector time (t_j - start) + delay_d + jitter (LIGO-T2100224), the
//      marginalised lnL and a logsumexp weighted by prior(t_j) delta_tc.
// float64 throughout.
// ---------------------------------------------------------------------------
template <int D>
__global__ void __launch_bounds__(kTmThreads) k_roq_time_marg(LaunchArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ double red[2 * kTmThreads];
  __shared__ long long s_rows[2 * kMaxDet];
  const int nl = a.roq_nl, nq = a.roq_nq;
  const int64_t n = a.roq_tm_n, max_rows = a.roq_tm_rows;
  double2* s_h = reinterpret_cast<double2*>(smem);  // [D][nl]
  double2* s_D = s_h + (size_t)D * nl;              // [D][max_rows], the current chunk's rows
  // roq.py:624-625: the weight grid's first time and spacing
  const double t0 = (double)a.roq_time_start * a.roq_dt;
  const double space = (double)(a.roq_time_start + 1) * a.roq_dt - t0;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, n_warps = blockDim.x >> 5;
  // every point, or (the recomputation of a mixed launch) the listed ones
  const int64_t n_items = a.rf_list_only ? (int64_t)*a.rf_count : a.B;
  for (int64_t it = blockIdx.x; it < n_items; it += gridDim.x) {
    const int64_t i = a.rf_list_only ? (int64_t)a.rf_list[it] : it;
    const PointRec& r = a.rec[i];
    const double jit = r.jitter;
    const bool tf2 = a.model == GWL_MODEL_TAYLORF2;
    const double u = tf2 ? cbrt(kPi * r.m_sec) : 0.0, lnu = tf2 ? log(u) : 0.0;
    const double pu5 = tf2 ? 3.0 / (128.0 * r.eta) / (u * u * u * u * u) : 0.0;
    double hh_part = 0.0;
    for (int q = threadIdx.x; q < nl; q += blockDim.x) {
      double2 hp = make_double2(0.0, 0.0), hx = make_double2(0.0, 0.0);
      const double f = a.roq_fl[q];
      const bool on = r.valid && (tf2 ? tf2_pols_t(a, r, a.roq_pl[q], f, u, lnu, pu5, hp, hx)
                                      : plain_pols(a, r, f, hp, hx));
#pragma unroll
      for (int d = 0; d < D; ++d) {
        const double hr = on ? hp.x * r.fp[d] + hx.x * r.fx[d] : 0.0;
        const double hi = on ? hp.y * r.fp[d] + hx.y * r.fx[d] : 0.0;
        s_h[(size_t)d * nl + q] = make_double2(hr, -hi);
      }
    }
    for (int q = threadIdx.x; q < nq; q += blockDim.x) {
      double2 hp = make_double2(0.0, 0.0), hx = make_double2(0.0, 0.0);
      const double f = a.roq_fq[q];
      if (!(r.valid && (tf2 ? tf2_pols_t(a, r, a.roq_pq[q], f, u, lnu, pu5, hp, hx) : plain_pols(a, r, f, hp, hx))))
        continue;
#pragma unroll
      for (int d = 0; d < D; ++d) {
        const double hr = hp.x * r.fp[d] + hx.x * r.fx[d], hi = hp.y * r.fp[d] + hx.y * r.fx[d];
        hh_part += (hr * hr + hi * hi) * a.roq_wq[d][q];
      }
    }
    const double hh = block_sum(hh_part, red);  // ends with a barrier: s_h is complete
    if (a.tm_series && a.hh_out && threadIdx.x == 0) a.hh_out[i] = hh;
    const double sr = r.dist / a.ref_dist, hh_ref = hh * r.dist * r.dist / (a.ref_dist * a.ref_dist);
    const double prob = 1.0 / (a.t_max - a.t_min);
    double m = -INFINITY, acc = 0.0;
    // the time samples in chunks, each with the weight rows its detector times read
    for (int64_t j0 = 0; j0 < n; j0 += a.roq_tm_chunk) {
      const int64_t j1 = (j0 + a.roq_tm_chunk < n ? j0 + a.roq_tm_chunk : n) - 1;
      if (threadIdx.x < D) {
        // the detector time grows with j: the rows of the chunk's first and last sample
        const int d = threadIdx.x;
        const double x0 = ((a.roq_tm_times[j0] - a.det[d].start_time) + r.dt[d]) + jit;
        const double x1 = ((a.roq_tm_times[j1] - a.det[d].start_time) + r.dt[d]) + jit;
        long long lo = (long long)floor((x0 - t0) / space) - 2, hi = (long long)floor((x1 - t0) / space) + 2;
        lo = lo < 0 ? 0 : lo;
        hi = hi > a.roq_n_time - 1 ? a.roq_n_time - 1 : hi;
        if (hi - lo + 1 > max_rows) hi = lo + max_rows - 1;
        s_rows[2 * d] = lo;
        s_rows[2 * d + 1] = hi >= lo ? hi - lo + 1 : 0;
      }
      __syncthreads();
#pragma unroll
      for (int d = 0; d < D; ++d) {
        const long long lo = s_rows[2 * d], nr = s_rows[2 * d + 1];
        for (long long k = warp; k < nr; k += n_warps) {
          const double2* w = a.roq_wl[d] + (size_t)(lo + k) * nl;
          const double2* h = s_h + (size_t)d * nl;
          double ar = 0.0, ai = 0.0;
          for (int q = lane; q < nl; q += 32) {
            const double2 wv = w[q], hv = h[q];
            ar += wv.x * hv.x - wv.y * hv.y;
            ai += wv.x * hv.y + wv.y * hv.x;
          }
#pragma unroll
          for (int o = 16; o > 0; o >>= 1) {
            ar += __shfl_xor_sync(0xffffffffu, ar, o);
            ai += __shfl_xor_sync(0xffffffffu, ai, o);
          }
          if (lane == 0) s_D[(size_t)d * max_rows + k] = make_double2(ar, ai);
        }
      }
      __syncthreads();
      for (int64_t j = j0 + threadIdx.x; j <= j1; j += blockDim.x) {
        const double tj = a.roq_tm_times[j];
        const double t = tj + jit;
        const bool in_prior = t >= a.t_min && t <= a.t_max;
        if (!in_prior && !a.tm_series) continue;
        double xr = 0.0, xi = 0.0;
        bool ok = true;
#pragma unroll
        for (int d = 0; d < D; ++d) {
          const double x = ((tj - a.det[d].start_time) + r.dt[d]) + jit;
          const double tpr = (x - t0) / space;
          const double fc = floor(tpr);
          const long long k = (long long)fc - s_rows[2 * d] - 2;
          if (k < 0 || k + 4 >= s_rows[2 * d + 1]) {
            ok = false;  // outside the weight grid
            continue;
          }
          const double2* Dd = s_D + (size_t)d * max_rows + k;
          const double2 m2 = Dd[0], m1 = Dd[1], c0 = Dd[2], p1 = Dd[3], p2 = Dd[4];
          const double b = tpr - fc, a1 = 1.0 - b;
          const double c = (a1 * a1 * a1 - a1) / 6.0, dd = (b * b * b - b) / 6.0;
          const double r1r = (-m2.x + 8.0 * m1.x - 14.0 * c0.x + 8.0 * p1.x - p2.x) / 4.0;
          const double r1i = (-m2.y + 8.0 * m1.y - 14.0 * c0.y + 8.0 * p1.y - p2.y) / 4.0;
          const double r2r = c0.x - 2.0 * p1.x + p2.x, r2i = c0.y - 2.0 * p1.y + p2.y;
          xr += a1 * c0.x + b * p1.x + c * r1r + dd * r2r;
          xi += a1 * c0.y + b * p1.y + c * r1i + dd * r2i;
        }
        if (a.tm_series) {
          // d_inner_h_array of roq.py:535-541 at every sample (NaN outside the weight grid)
          reinterpret_cast<double2*>(a.tm_series)[(size_t)i * n + j] =
              ok ? make_double2(xr, xi) : make_double2(NAN, NAN);
          if (!in_prior) continue;
        }
        double l;
        const double pw = a.tm_prior ? tm_prior_density(a, t) : 1.0;  // base.py:807, prior(t_j)
        if (!ok || !(pw > 0.0)) {
          l = -INFINITY;
        } else if (a.dist_marg) {
          const double dx = a.phase_marg ? sqrt(xr * xr + xi * xi) * sr : xr * sr;
          l = bicubic_eval(a.tx, a.nx, a.ty, a.ny, a.tc, a.bbox, dx, hh_ref);
        } else if (a.phase_marg) {
          l = ln_i0(sqrt(xr * xr + xi * xi)) - hh / 2;
        } else {
          l = xr - hh / 2;
        }
        if (a.tm_prior && isfinite(l)) l += log(pw);
        if (l > m) {
          acc = isfinite(m) ? acc * exp(m - l) + 1.0 : 1.0;
          m = l;
        } else if (isfinite(l)) {
          acc += exp(l - m);
        }
      }
      __syncthreads();  // s_rows and s_D are rewritten by the next chunk
    }
    // combine the (m, acc) pairs in a fixed tree order
    double* redm = red;
    double* reds = red + kTmThreads;
    redm[threadIdx.x] = m;
    reds[threadIdx.x] = acc;
    __syncthreads();
    for (int w = kTmThreads / 2; w > 0; w >>= 1) {
      if (threadIdx.x < w) {
        const double m1 = redm[threadIdx.x], m2 = redm[threadIdx.x + w];
        const double s1 = reds[threadIdx.x], s2 = reds[threadIdx.x + w];
        const double mm = fmax(m1, m2);
        double ss = 0.0;
        if (isfinite(mm)) ss = (isfinite(m1) ? s1 * exp(m1 - mm) : 0.0) + (isfinite(m2) ? s2 * exp(m2 - mm) : 0.0);
        redm[threadIdx.x] = mm;
        reds[threadIdx.x] = ss;
      }
      __syncthreads();
    }
    if (threadIdx.x == 0) {
      const double amax = redm[0], total = reds[0] * (a.tm_prior ? 1.0 : prob) * a.delta_tc;
      double lnl;
      if (!r.valid) lnl = -1.7976931348623157e308;
      else if (!isfinite(amax)) lnl = amax;
      else lnl = amax + log(total);
      a.out[i] = lnl;
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// ROQ with time marginalisation, mixed precision.  Step 2 of the float64
// kernel, D_d[k] = sum_q W_d[k][q] conj(h_d(F_q)), is a matrix product over
// the batch: (weight rows x linear nodes) x (linear nodes x points) per
// detector.  It runs as complex float32 GEMMs over every row of the weight
// grid (cuBLAS, pedantic float32 math: no reduced-precision tensor path),
// one per group of kRoqSplits consecutive node groups (a strided batch), so
// that each float32 sum has a few tens of terms; around them
//   k_roq_nodes32: conj(h_d) at the linear nodes from the float64 model,
//     stored as float32 pairs (zero in the padding), with <h|h> (float64,
//     quadratic nodes);
//   k_roq_tm_mixed: per point, the groups' partial rows summed in
//     float-float (TwoSum) into shared memory over the rows the point reads,
//     the five-sample interpolation at each marginalisation sample's detector
//     time, the per-sample marginalised lnL and the logsumexp in float32 (the
//     large terms in float64).  The detector time's index on the weight grid
//     is the float64 value of the float64 kernel split into integer and
//     fraction parts on the host (per sample) and once per point (per
//     detector), so that no float64 arithmetic runs per sample.
// Error bound of a point (|dlnL| <= s |dX|, s = tm_sensitivity): the float32
// rounding of each group's products and sums, below kRoqErrNorm times
// C_d = (sum_s (max_k ||W_dk,s||_2 ||h_d,s||_2)^2)^(1/2) per detector (the
// groups' errors are independent; a K-term float32 dot product errs by about
// u ||w|| ||h|| / sqrt(2) when summed in order), and the rounding of the
// summed rows and the interpolation, below kRoqErrPeak max_j |X_j|.  On the
// 400-node empirical-interpolation basis of the benchmark (8192 prior draws
// with time, and with time and phase marginalisation) the largest |dlnL| was
// 0.18 of this bound with the coefficient 6 u; kRoqErrNorm = 3 u keeps a
// margin of 2.7.  Points over the tolerance are listed for the float64 kernel.
// ---------------------------------------------------------------------------
constexpr double kRoqErrNorm = 3.0 * 5.9604644775390625e-08;
constexpr double kRoqErrPeak = 1e-6;
constexpr int kRoqNodeThreads = 128;
constexpr int kRoqMixThreads = 256;

template <int D>
__global__ void __launch_bounds__(kRoqNodeThreads) k_roq_nodes32(LaunchArgs a) {
  __shared__ double red[kRoqNodeThreads / 32];
  const int64_t p = blockIdx.x, i = a.roq_c0 + p, cn = a.roq_cn;
  const int nl = a.roq_nl, nq = a.roq_nq, np = a.roq_nl_pad;
  const PointRec& r = a.rec[i];
  const bool tf2 = a.model == GWL_MODEL_TAYLORF2;
  const double u = tf2 ? cbrt(kPi * r.m_sec) : 0.0, lnu = tf2 ? log(u) : 0.0;
  const double pu5 = tf2 ? 3.0 / (128.0 * r.eta) / (u * u * u * u * u) : 0.0;
  for (int q = threadIdx.x; q < np; q += blockDim.x) {
    double2 hp = make_double2(0.0, 0.0), hx = make_double2(0.0, 0.0);
    const bool on = q < nl && r.valid &&
                    (tf2 ? tf2_pols_t(a, r, a.roq_pl[q], a.roq_fl[q], u, lnu, pu5, hp, hx)
                         : plain_pols(a, r, a.roq_fl[q], hp, hx));
#pragma unroll
    for (int d = 0; d < D; ++d) {
      const double hr = on ? hp.x * r.fp[d] + hx.x * r.fx[d] : 0.0;
      const double hi = on ? hp.y * r.fp[d] + hx.y * r.fx[d] : 0.0;
      a.roq_h32[((size_t)d * cn + p) * np + q] = make_float2((float)hr, (float)-hi);
    }
  }
  double hh_part = 0.0;
  for (int q = threadIdx.x; q < nq; q += blockDim.x) {
    double2 hp = make_double2(0.0, 0.0), hx = make_double2(0.0, 0.0);
    const double f = a.roq_fq[q];
    if (!(r.valid && (tf2 ? tf2_pols_t(a, r, a.roq_pq[q], f, u, lnu, pu5, hp, hx) : plain_pols(a, r, f, hp, hx))))
      continue;
#pragma unroll
    for (int d = 0; d < D; ++d) {
      const double hr = hp.x * r.fp[d] + hx.x * r.fx[d], hi = hp.y * r.fp[d] + hx.y * r.fx[d];
      hh_part += (hr * hr + hi * hi) * a.roq_wq[d][q];
    }
  }
  // a fixed-order sum: xor-shuffles within the warps, then the warps in order
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) hh_part += __shfl_xor_sync(0xffffffffu, hh_part, o);
  if (lane == 0) red[warp] = hh_part;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < kRoqNodeThreads / 32; ++w) t += red[w];
    a.roq_hh[p] = t;
  }
}

// rows of detector d the samples [j0, j1) read: grid indices from
// floor(g_j) + b_d - 2 to floor(g_j) + b_d + 1 + 2, clamped to the grid
__device__ __forceinline__ void roq_row_range(const LaunchArgs& a, int64_t j0, int64_t j1, int bi, int64_t* lo,
                                              int64_t* n) {
  const int64_t nt = a.roq_n_time;
  if (j1 <= j0) {
    *lo = 0;
    *n = 0;
    return;
  }
  int64_t k0 = (int64_t)a.roq_tm_g[j0].x + bi - 2, k1 = (int64_t)a.roq_tm_g[j1 - 1].x + bi + 3;
  k0 = k0 < 0 ? 0 : k0;
  k1 = k1 > nt - 1 ? nt - 1 : k1;
  *lo = k0;
  *n = k1 >= k0 ? k1 - k0 + 1 : 0;
}

template <int D>
__global__ void __launch_bounds__(kRoqMixThreads) k_roq_tm_mixed(LaunchArgs a) {
  // dynamic shared memory: the distance spline's knots tx [nx], ty [ny], then
  // per detector the summed rows the point reads (float32 pairs, nt at most)
  extern __shared__ __align__(16) float s_dyn[];
  __shared__ SplineRowF s_row;
  __shared__ float redf[3 * (kRoqMixThreads / 32)];
  __shared__ float s_hn[kMaxDet * kRoqSplits];
  __shared__ double s_scal[2];
  __shared__ int s_bi[kMaxDet];
  __shared__ float s_bf[kMaxDet];
  __shared__ long long s_j[2], s_klo[kMaxDet], s_kn[kMaxDet];
  const int64_t p = blockIdx.x, i = a.roq_c0 + p, cn = a.roq_cn, nt = a.roq_n_time;
  const PointRec& r = a.rec[i];
  float* s_tx = s_dyn;
  float* s_ty = s_dyn + a.nx;
  const int kn0 = a.dist_marg ? ((a.nx + a.ny + 3) & ~3) : 0;
  float2* s_rows = reinterpret_cast<float2*>(s_dyn + kn0);  // [D][nt]
  if (a.dist_marg) {
    for (int q = threadIdx.x; q < a.nx; q += blockDim.x) s_tx[q] = a.tx_f[q];
    for (int q = threadIdx.x; q < a.ny; q += blockDim.x) s_ty[q] = a.ty_f[q];
  }
  const double jit = r.jitter;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  constexpr int W = kRoqMixThreads / 32;
  if (threadIdx.x == 0) {
    s_scal[0] = a.roq_hh[p];
    s_scal[1] = r.dist / a.ref_dist;
    // the samples inside the prior: t_j + jit in [t_min, t_max], tested as
    // the float64 kernel tests them (the times increase)
    const int64_t n = a.roq_tm_n;
    int64_t lo = 0, hi = n;
    while (lo < hi) {
      const int64_t mid = (lo + hi) / 2;
      if (a.roq_tm_times[mid] + jit >= a.t_min) hi = mid; else lo = mid + 1;
    }
    int64_t lo2 = lo, hi2 = n;  // first sample past t_max
    while (lo2 < hi2) {
      const int64_t mid = (lo2 + hi2) / 2;
      if (a.roq_tm_times[mid] + jit <= a.t_max) lo2 = mid + 1; else hi2 = mid;
    }
    s_j[0] = lo;
    s_j[1] = lo2;
  }
  if (threadIdx.x >= 32 && threadIdx.x < 32 + D) {
    // detector d's grid index offset ((start_0 - start_d) + dt_d + jit) / dt, split
    const int d = threadIdx.x - 32;
    const double t0 = (double)a.roq_time_start * a.roq_dt;
    const double space = (double)(a.roq_time_start + 1) * a.roq_dt - t0;
    const double bd = (((a.det[0].start_time - a.det[d].start_time) + r.dt[d]) + jit) / space;
    const double fb = floor(bd);
    s_bi[d] = (int)fb;
    s_bf[d] = (float)(bd - fb);
  }
  // ||h_d,s||_2 per node group, one warp per (detector, group), fixed order
  for (int ds = warp; ds < D * kRoqSplits; ds += W) {
    const int d = ds / kRoqSplits, sp = ds % kRoqSplits;
    const float2* h = a.roq_h32 + ((size_t)d * cn + p) * a.roq_nl_pad + (size_t)sp * a.roq_ks;
    float n2 = 0.f;
    for (int q = lane; q < a.roq_ks; q += 32) n2 = __fmaf_rn(h[q].x, h[q].x, __fmaf_rn(h[q].y, h[q].y, n2));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) n2 += __shfl_xor_sync(0xffffffffu, n2, o);
    if (lane == 0) s_hn[ds] = sqrtf(n2);
  }
  __syncthreads();
  if (threadIdx.x < D) {
    int64_t lo, n;
    roq_row_range(a, s_j[0], s_j[1], s_bi[threadIdx.x], &lo, &n);
    s_klo[threadIdx.x] = lo;
    s_kn[threadIdx.x] = n;
  }
  const double hh = s_scal[0], sr = s_scal[1];
  if (threadIdx.x == 32 && a.dist_marg) s_row = bicubic_row_f(s_ty, a.ny, a.bbox, (float)(hh * sr * sr));
  __syncthreads();
  // the groups' partial rows summed in float-float, rounded once to float32
#pragma unroll
  for (int d = 0; d < D; ++d) {
    const int64_t klo = s_klo[d], kn = s_kn[d];
    const float2* src = a.roq_d32 + ((size_t)d * kRoqSplits * cn + p) * nt + klo;
    for (int64_t k = threadIdx.x; k < kn; k += blockDim.x) {
      float xh = 0.f, xl = 0.f, yh = 0.f, yl = 0.f;
#pragma unroll
      for (int sp = 0; sp < kRoqSplits; ++sp) {
        const float2 v = src[(size_t)sp * cn * nt + k];
        two_sum_acc(xh, xl, v.x);
        two_sum_acc(yh, yl, v.y);
      }
      s_rows[(size_t)d * nt + k] = make_float2(__fadd_rn(xh, xl), __fadd_rn(yh, yl));
    }
  }
  __syncthreads();
  double m = -INFINITY, acc = 0.0;
  float xmax = 0.f;
  const int64_t j1 = s_j[1];
  for (int64_t j = s_j[0] + threadIdx.x; j < j1; j += blockDim.x) {
    const int2 g = a.roq_tm_g[j];
    const float gf = __int_as_float(g.y);
    float xr = 0.f, xi = 0.f;
    bool ok = true;
#pragma unroll
    for (int d = 0; d < D; ++d) {
      // grid index fc = floor(g + b_d) and fraction b, rows fc - 2 .. fc + 2
      const float sf = gf + s_bf[d];
      const int carry = sf >= 1.f ? 1 : 0;
      const float b = sf - (float)carry;
      const int64_t k = (int64_t)g.x + s_bi[d] + carry - 2;
      if (k < 0 || k + 4 > nt - 1) {
        ok = false;  // outside the weight grid
        continue;
      }
      const float2* Dd = s_rows + (size_t)d * nt + (k - s_klo[d]);
      const float2 m2 = Dd[0], m1 = Dd[1], c0 = Dd[2], p1 = Dd[3], p2 = Dd[4];
      const float a1 = 1.f - b;
      const float c = (a1 * a1 * a1 - a1) * (1.f / 6.f), dd = (b * b * b - b) * (1.f / 6.f);
      const float r1r = (-m2.x + 8.f * m1.x - 14.f * c0.x + 8.f * p1.x - p2.x) * 0.25f;
      const float r1i = (-m2.y + 8.f * m1.y - 14.f * c0.y + 8.f * p1.y - p2.y) * 0.25f;
      const float r2r = c0.x - 2.f * p1.x + p2.x, r2i = c0.y - 2.f * p1.y + p2.y;
      xr += a1 * c0.x + b * p1.x + c * r1r + dd * r2r;
      xi += a1 * c0.y + b * p1.y + c * r1i + dd * r2i;
    }
    if (!ok) continue;
    double lw = 0.0;
    if (a.tm_prior) {
      const float pw = tm_prior_density_f(a, a.roq_tm_times[j] + jit);  // base.py:807, prior(t_j)
      if (!(pw > 0.f)) continue;
      lw = (double)__logf(pw);
    }
    const double l = tm_lnl_mixed(a, xr, xi, hh, sr, s_tx, s_row) + lw;
    xmax = fmaxf(xmax, sqrtf(xr * xr + xi * xi));
    tm_lse_push<true>(l, m, acc);
  }
  // the block's logsumexp: the float32 maximum of the threads' m (any
  // reference near the maximum serves), then sum acc_t exp(m_t - M), both by
  // xor-shuffles within warps and a fixed-order sum over the warps
  float mf = (float)m, xm = xmax;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    mf = fmaxf(mf, __shfl_xor_sync(0xffffffffu, mf, o));
    xm = fmaxf(xm, __shfl_xor_sync(0xffffffffu, xm, o));
  }
  if (lane == 0) {
    redf[warp] = mf;
    redf[W + warp] = xm;
  }
  __syncthreads();
  float M = redf[0];
  for (int w = 1; w < W; ++w) M = fmaxf(M, redf[w]);
  float sm = 0.f;
  if (isfinite(M) && isfinite(m)) sm = (float)acc * __expf((float)(m - (double)M));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) sm += __shfl_xor_sync(0xffffffffu, sm, o);
  if (lane == 0) redf[2 * W + warp] = sm;
  __syncthreads();
  if (threadIdx.x == 0) {
    float total = 0.f, xp = 0.f;
    for (int w = 0; w < W; ++w) {
      total += redf[2 * W + w];
      xp = fmaxf(xp, redf[W + w]);
    }
    const double prob = 1.0 / (a.t_max - a.t_min);
    const double tot = (double)total * (a.tm_prior ? 1.0 : prob) * a.delta_tc;
    double lnl;
    if (!r.valid) lnl = -1.7976931348623157e308;
    else if (!isfinite(M)) lnl = (double)M;
    else lnl = (double)M + (double)logf((float)tot);
    a.out[i] = lnl;
    if (a.rf_tol > 0 && a.rf_count && a.rf_list && r.valid) {
      double gemm = 0.0;
      for (int d = 0; d < D; ++d) {
        double c2 = 0.0;
        for (int sp = 0; sp < kRoqSplits; ++sp) {
          const double c = (double)a.roq_wnorm[d][sp] * (double)s_hn[d * kRoqSplits + sp];
          c2 += c * c;
        }
        gemm += sqrt(c2);
      }
      const double err =
          tm_sensitivity(a, (double)xp, sr, s_tx, s_row) * (kRoqErrNorm * gemm + kRoqErrPeak * (double)xp);
      if (!(err <= a.rf_tol)) a.rf_list[atomicAdd(a.rf_count, 1)] = (int32_t)i;
    }
  }
}

size_t roq_tm_mixed_smem(const LaunchArgs& a) {
  const size_t knots = a.dist_marg ? (size_t)((a.nx + a.ny + 3) & ~3) * sizeof(float) : 0;
  return knots + (size_t)a.n_det * (size_t)a.roq_n_time * sizeof(float2);
}

bool roq_tm_mixed_fits(const LaunchArgs& a) { return roq_tm_mixed_smem(a) <= (size_t)200 * 1024; }

template <int D>
static cudaError_t launch_roq_nodes32_d(const LaunchArgs& a, cudaStream_t s) {
  k_roq_nodes32<D><<<(unsigned)a.roq_cn, kRoqNodeThreads, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_roq_nodes32(const LaunchArgs& a, cudaStream_t s) {
  if (a.roq_cn < 1) return cudaSuccess;
  switch (a.n_det) {
    case 1: return launch_roq_nodes32_d<1>(a, s);
    case 2: return launch_roq_nodes32_d<2>(a, s);
    case 3: return launch_roq_nodes32_d<3>(a, s);
    default: return launch_roq_nodes32_d<4>(a, s);
  }
}

template <int D>
static cudaError_t launch_roq_tm_mixed_d(const LaunchArgs& a, cudaStream_t s) {
  const size_t smem = roq_tm_mixed_smem(a);  // the opt-in covers the dynamic part
  const cudaError_t e =
      cudaFuncSetAttribute(k_roq_tm_mixed<D>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  k_roq_tm_mixed<D><<<(unsigned)a.roq_cn, kRoqMixThreads, smem, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_roq_tm_mixed(const LaunchArgs& a, cudaStream_t s) {
  if (a.roq_cn < 1) return cudaSuccess;
  if (!roq_tm_mixed_fits(a)) return cudaErrorInvalidValue;  // checked on the host first
  switch (a.n_det) {
    case 1: return launch_roq_tm_mixed_d<1>(a, s);
    case 2: return launch_roq_tm_mixed_d<2>(a, s);
    case 3: return launch_roq_tm_mixed_d<3>(a, s);
    default: return launch_roq_tm_mixed_d<4>(a, s);
  }
}

// exp(-2 pi i t / L), t < L / 2, in float64 and float32, one table per
// (device, FFT length), kept for the life of the process: analyses of
// different lengths may launch at the same time from different host threads,
// so a table is never replaced or freed while a kernel may read it, and the
// tables of one device are never handed to a launch on another.
namespace {
PerDeviceCache<TwiddleTables> g_twiddles;
}  // namespace

cudaError_t twiddles_for(int64_t L, TwiddleTables* out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const int rc = g_twiddles.get(dev, L, out, [L](TwiddleTables* t) -> int {
    const int64_t H = L / 2;
    double2* h64 = new double2[H];
    float2* h32 = new float2[H];
    for (int64_t q = 0; q < H; ++q) {
      // exp(-2 pi i q / L), argument reduced to an exact rational of pi
      const double ang = -2.0 * 3.141592653589793 * (double)q / (double)L;
      h64[q] = make_double2(std::cos(ang), std::sin(ang));
      h32[q] = make_float2((float)h64[q].x, (float)h64[q].y);
    }
    cudaError_t err = cudaMalloc(&t->d64, H * sizeof(double2));
    if (err == cudaSuccess) err = cudaMalloc(&t->d32, H * sizeof(float2));
    if (err == cudaSuccess) err = cudaMemcpy(t->d64, h64, H * sizeof(double2), cudaMemcpyHostToDevice);
    if (err == cudaSuccess) err = cudaMemcpy(t->d32, h32, H * sizeof(float2), cudaMemcpyHostToDevice);
    delete[] h64;
    delete[] h32;
    if (err != cudaSuccess) {
      cudaFree(t->d64);
      cudaFree(t->d32);
      return (int)err;
    }
    return 0;
  });
  return static_cast<cudaError_t>(rc);
}

namespace {

int tm_grid_fp64() {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return sms > 0 ? 2 * sms : 304;
}

}  // namespace

bool fft_length_supported(int64_t L, int* m_odd, int* log2N) {
  if (L < 16) return false;
  int64_t m = L;
  int p = 0;
  while ((m & 1) == 0) {
    m >>= 1;
    ++p;
  }
  if (p < 4 || m > kTmMaxOddFactor) return false;
  *m_odd = (int)m;
  *log2N = p;
  return true;
}

size_t time_marg_work_bytes(const LaunchArgs& a) {
  // float64 integrand / FFT slots, one per resident CTA
  return (size_t)tm_grid_fp64() * (size_t)a.n_fft * sizeof(double2);
}

// shared memory of k_tm_half: the half-length buffer, the window's values, the spline's knots
static size_t tm_half_smem(const LaunchArgs& a, int* n_win_cap) {
  const double width = (a.t_max - a.t_min) / a.tm_step;
  *n_win_cap = (int)std::ceil(width > 0.0 && width < 1e7 ? width : 0.0) + 8;
  const int64_t M = a.n_fft >> kTmHalfLs;
  return (size_t)(M + M / 16) * sizeof(float2) + (size_t)*n_win_cap * sizeof(float2) +
         (a.dist_marg ? (size_t)(a.nx + a.ny) * sizeof(float) : 0);
}

template <int D>
static cudaError_t launch_tm_d(const LaunchArgs& a, cudaStream_t s, int log2N, int m_odd, const TwiddleTables& tw) {
  int n_win_cap = 0;
  if (a.precision == GWL_PRECISION_MIXED && a.model == GWL_MODEL_TAYLORF2 && m_odd == 1 && log2N >= 5 + kTmHalfLs &&
      tm_half_smem(a, &n_win_cap) <= ((size_t)200 * 1024 >> kTmHalfLs)) {
    // 2^kTmHalfLs shorter transforms per point, as many CTAs per SM
    const size_t smem = tm_half_smem(a, &n_win_cap);
    cudaError_t e =
        cudaFuncSetAttribute(k_tm_half<D, kTmHalfLs>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k_tm_half<D, kTmHalfLs><<<(unsigned)a.B, 512 >> kTmHalfLs, smem, s>>>(a, tw.d32, log2N, n_win_cap);
    return cudaGetLastError();
  }
  if (a.precision == GWL_PRECISION_MIXED) {
    // the FFT buffer, then the distance spline's knots
    const size_t smem = (size_t)(a.n_fft + a.n_fft / 16) * sizeof(float2) +
                        (a.dist_marg ? (size_t)(a.nx + a.ny) * sizeof(float) : 0);
    cudaError_t e = cudaFuncSetAttribute(k_time_marg<D, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    const unsigned grid = (unsigned)a.B;
    k_time_marg<D, true><<<grid, kTmThreads, smem, s>>>(a, tw.d32, log2N, m_odd);
  } else {
    // relative binning: the edge ratios in shared memory
    const size_t smem = a.relbin ? (size_t)a.rb_edges * D * sizeof(double2) : 0;
    if (smem > 0) {  // static and dynamic together may pass 48 KB
      cudaError_t e =
          cudaFuncSetAttribute(k_time_marg<D, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
    }
    const unsigned grid = (unsigned)std::min<int64_t>(a.B, tm_grid_fp64());
    k_time_marg<D, false><<<grid, kTmThreads, smem, s>>>(a, tw.d64, log2N, m_odd);
  }
  return cudaGetLastError();
}

size_t roq_time_marg_smem(const LaunchArgs& a) {
  return (size_t)a.n_det * ((size_t)a.roq_nl + (size_t)a.roq_tm_rows) * sizeof(double2);
}

template <int D>
static cudaError_t launch_roq_tm_d(const LaunchArgs& a, cudaStream_t s) {
  // the opt-in covers the dynamic part; static and dynamic together may pass 48 KB
  const size_t smem = roq_time_marg_smem(a);
  cudaError_t e = cudaFuncSetAttribute(k_roq_time_marg<D>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  const unsigned grid = (unsigned)std::min<int64_t>(a.B, 4 * (int64_t)tm_grid_fp64());
  k_roq_time_marg<D><<<grid, kTmThreads, smem, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_roq_time_marginalized(const LaunchArgs& a, cudaStream_t s) {
  // checked on the host first
  if (roq_time_marg_smem(a) > 200 * 1024 || a.roq_tm_n < 1 || a.roq_tm_chunk < 1 || a.roq_tm_rows < 5)
    return cudaErrorInvalidValue;
  switch (a.n_det) {
    case 1: return launch_roq_tm_d<1>(a, s);
    case 2: return launch_roq_tm_d<2>(a, s);
    case 3: return launch_roq_tm_d<3>(a, s);
    default: return launch_roq_tm_d<4>(a, s);
  }
}

cudaError_t launch_time_marginalized(const LaunchArgs& a, cudaStream_t s) {
  int m_odd = 0, log2N = 0;
  if (!fft_length_supported(a.n_fft, &m_odd, &log2N)) return cudaErrorInvalidValue;  // checked on the host first
  if (a.precision != GWL_PRECISION_MIXED && a.relbin && (size_t)a.rb_edges * a.n_det * sizeof(double2) > 200 * 1024)
    return cudaErrorInvalidValue;  // the host checks the edge count first
  if (a.precision == GWL_PRECISION_MIXED &&
      ((size_t)(a.n_fft + a.n_fft / 16) * sizeof(float2) + (a.dist_marg ? (size_t)(a.nx + a.ny) * sizeof(float) : 0) >
           200 * 1024 ||
                                             a.n_fft / 2 > (int64_t)kTmTwiddleRows * kTmTwiddleRows))
    return cudaErrorInvalidValue;
  TwiddleTables tw;
  cudaError_t e = twiddles_for(a.n_fft, &tw);
  if (e != cudaSuccess) return e;
  switch (a.n_det) {
    case 1: return launch_tm_d<1>(a, s, log2N, m_odd, tw);
    case 2: return launch_tm_d<2>(a, s, log2N, m_odd, tw);
    case 3: return launch_tm_d<3>(a, s, log2N, m_odd, tw);
    default: return launch_tm_d<4>(a, s, log2N, m_odd, tw);
  }
}

}  // namespace gwl
