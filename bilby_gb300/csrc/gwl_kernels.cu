// Likelihood kernels: per-point prologue, fused float64 ("plain") kernels,
// fused mixed-precision kernels and the per-point finalize step.
//
// Layout: one thread per parameter point (128 points per CTA), the CTA walks
// one chunk of frequency bins whose data / PSD / basis tables are staged in
// shared memory once and read by all 128 points (broadcast loads).  Partial
// sums per (chunk, point, detector) go to a work buffer and are reduced in a
// fixed order by the finalize kernel, so a point's result does not depend on
// which other points share its batch.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>

#include "gwl_device.cuh"
#include "gwl_internal.h"
#include "gwl_math.cuh"

namespace gwl {

__device__ __forceinline__ double par(const LaunchArgs& a, int slot, int64_t i) {
  return a.params[(int64_t)slot * a.B + i];
}

// ---------------------------------------------------------------------------
// prologue: per-point float64 set-up (sky frame, antenna, delays, model scalars)
// ---------------------------------------------------------------------------
__global__ void k_prologue(LaunchArgs a) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.B) return;
  PointRec r;
  memset(&r, 0, sizeof(r));
  const double ra = par(a, GWL_P_RA, i), dec = par(a, GWL_P_DEC, i), psi = par(a, GWL_P_PSI, i);
  double tgeo = par(a, GWL_P_GEOCENT_TIME, i);
  r.jitter = a.time_marg && a.jitter ? par(a, GWL_P_TIME_JITTER, i) : 0.0;
  // base.py:427-428: the jitter is added to geocent_time before projection.
  tgeo = tgeo + r.jitter;
  const double gmst = pymod(gmst_radians(tgeo), kTwoPi);
  bool ok = isfinite(ra) && isfinite(dec) && isfinite(psi) && isfinite(tgeo);
  for (int d = 0; d < a.n_det; ++d) {
    double fp, fx, delay;
    antenna_and_delay(a.det[d].tensor, a.det[d].vertex, ra, dec, psi, gmst, &fp, &fx, &delay);
    r.fp[d] = fp;
    r.fx[d] = fx;
    // interferometer.py:355-358: subtract the two GPS times first, then add the delay.
    const double dt_geocent = tgeo - a.det[d].start_time;
    r.dt[d] = dt_geocent + delay;
    // frac(dt * df) in cycles per bin as 0.64 fixed point, so that the phase
    // 2 pi f_k dt = 2 pi k (dt df) reduces exactly modulo one cycle.
    const double x = r.dt[d] * a.step;
    const double frac = x - floor(x);
    double scaled = ldexp(frac, 64);
    if (!(scaled < 18446744073709551616.0)) scaled = 0.0;
    const unsigned long long u = (unsigned long long)scaled;
    r.xfix[d][0] = (uint32_t)(u & 0xffffffffull);
    r.xfix[d][1] = (uint32_t)(u >> 32);
  }
  if (a.model == GWL_MODEL_SINEGAUSSIAN) {
    // bilby/gw/source.py:1197-1207
    const double hrss = par(a, GWL_P_HRSS, i), Q = par(a, GWL_P_Q, i), f0 = par(a, GWL_P_FREQUENCY, i);
    const double tau = Q / (1.4142135623730951 * kPi * f0);
    const double temp = Q / (4.0 * 1.7724538509055159 * f0);
    r.a[0] = hrss * 1.7724538509055159 * tau / 2;          // plus and cross prefactor
    r.a[1] = sqrt(temp * (1 + exp(-Q * Q)));                // plus denominator
    r.a[2] = sqrt(temp * (1 - exp(-Q * Q)));                // cross denominator
    r.a[3] = tau * tau;
    r.sg_f0 = f0;
    r.sg_a = 9.869604401089358 * tau * tau;  // pi^2 tau^2 for the mixed kernel
    r.amp = r.a[0] / r.a[1];
    r.amp2 = r.a[0] / r.a[2];
    ok = ok && isfinite(r.amp) && isfinite(r.amp2) && isfinite(r.sg_a) && f0 > 0;
  } else {
    const double m1 = par(a, GWL_P_MASS_1, i), m2 = par(a, GWL_P_MASS_2, i);
    const double chi1 = par(a, GWL_P_CHI_1, i), chi2 = par(a, GWL_P_CHI_2, i);
    const double dl = par(a, GWL_P_LUMINOSITY_DISTANCE, i);
    const double theta_jn = par(a, GWL_P_THETA_JN, i), phase = par(a, GWL_P_PHASE, i);
    const double m = m1 + m2;
    r.m_sec = m * kMtsunSI;
    r.eta = m1 * m2 / (m * m);
    r.f_isco = 1.0 / (6.0 * sqrt(6.0) * kPi * r.m_sec);
    const double mc_sec = pow(r.eta, 0.6) * m * kMtsunSI;
    r.dist = dl;
    r.amp = sqrt(5.0 / 24.0) * pow(kPi, -2.0 / 3.0) * pow(mc_sec, 5.0 / 6.0) * kSpeedOfLight / (dl * 1e6 * kPcSI);
    r.cos_i = cos(theta_jn);
    r.phase = phase;
    taylorf2_coefficients(m1, m2, chi1, chi2, r.a, r.l);
    ok = ok && m1 > 0 && m2 > 0 && dl > 0 && isfinite(r.amp) && isfinite(phase) && isfinite(chi1) &&
         isfinite(chi2);
    // band [k_start, k_end): f >= minimum_frequency and f < f_isco
    int64_t lo = 0, hi = a.n_bins;  // first k with freq[k] >= f_isco
    while (lo < hi) {
      const int64_t mid = (lo + hi) / 2;
      if (a.freq[mid] >= r.f_isco) hi = mid; else lo = mid + 1;
    }
    r.k_end = lo;
    r.k_start = a.k_fmin;
    // Psi / (2 pi) = sum_b c_b phi_b(f) + c_const with v = u f^(1/3), u = (pi M)^(1/3)
    const double P = 3.0 / (128.0 * r.eta) / kTwoPi;
    const double u = cbrt(kPi * r.m_sec);
    const double lnu = log(u);
    double c[kNumBasis];
    c[0] = P * r.a[0] / (u * u * u * u * u);   // f^(-5/3)
    c[1] = P * r.a[2] / (u * u * u);           // f^(-1)
    c[2] = P * r.a[3] / (u * u);               // f^(-2/3)
    c[3] = P * r.a[4] / u;                     // f^(-1/3)
    c[4] = P * r.l[5] / 3.0;                   // ln f
    c[5] = P * (r.a[6] + r.l[6] * lnu) * u;    // f^(1/3)
    c[6] = P * r.l[6] / 3.0 * u;               // f^(1/3) ln f
    c[7] = P * r.a[7] * u * u;                 // f^(2/3)
    const double cconst = P * (r.a[5] + r.l[5] * lnu) + (-2.0 * phase - kPi / 4) / kTwoPi;
    for (int b = 0; b < kNumBasis; ++b) {
      const ff s = ff_from_double(c[b]);
      r.c_hi[b] = s.hi;
      r.c_lo[b] = s.lo;
    }
    const ff s = ff_from_double(cconst - floor(cconst));
    r.c_hi[kNumBasis] = s.hi;
    r.c_lo[kNumBasis] = s.lo;
  }
  r.valid = ok ? 1 : 0;
  a.rec[i] = r;
}

// ---------------------------------------------------------------------------
// plain float64 kernels
// ---------------------------------------------------------------------------
template <int D>
__global__ void __launch_bounds__(kPointsPerCta) k_plain_sg(LaunchArgs a) {
  constexpr int CH = kChunkPlain;
  __shared__ double s_f[CH];
  __shared__ double2 s_d[D][CH];
  __shared__ double s_is[D][CH];
  const int64_t k0 = a.k_base + (int64_t)blockIdx.y * CH;
  for (int j = threadIdx.x; j < CH; j += blockDim.x) {
    const int64_t k = k0 + j;
    s_f[j] = a.freq[k];
#pragma unroll
    for (int d = 0; d < D; ++d) {
      s_d[d][j] = reinterpret_cast<const double2*>(a.strain[d])[k];
      s_is[d][j] = a.inv_psd[d][k];
    }
  }
  __syncthreads();
  const int64_t i = (int64_t)blockIdx.x * kPointsPerCta + threadIdx.x;
  if (i >= a.B) return;
  const PointRec& r = a.rec[i];
  double* out = a.part + (((int64_t)blockIdx.y * a.B + i) * D) * kPartStride;
  double dre[D], dim[D], hh[D], fp[D], fx[D], w2[D];
#pragma unroll
  for (int d = 0; d < D; ++d) {
    dre[d] = dim[d] = hh[d] = 0.0;
    fp[d] = r.fp[d];
    fx[d] = r.fx[d];
    w2[d] = 2.0 * kPi * r.dt[d];
  }
  if (r.valid) {
    const double f0 = r.sg_f0, amp = r.a[0], dplus = r.a[1], dcross = r.a[2], tau2 = r.a[3];
    const double pi2 = 9.869604401089358;
    for (int j = 0; j < CH; ++j) {
      const double f = s_f[j];
      // source.py:1199-1207
      const double fm = f - f0, fpl = f + f0;
      const double neg = exp(-(fm * fm) * pi2 * tau2);
      const double pos = exp(-(fpl * fpl) * pi2 * tau2);
      const double hp = amp * (neg + pos) / dplus;       // real
      const double hx_im = -(amp * (neg - pos) / dcross); // h_x = i * hx_im
#pragma unroll
      for (int d = 0; d < D; ++d) {
        const double is = s_is[d][j];
        if (is == 0.0) continue;
        // interferometer.py:341-362
        const double sre = hp * fp[d];
        const double sim = hx_im * fx[d];
        double sn, cs;
        sincos(w2[d] * f, &sn, &cs);  // exp(-i w f) = cs - i sn
        const double hre = sre * cs + sim * sn;
        const double him = sim * cs - sre * sn;
        const double2 dd = s_d[d][j];
        // utils.py:118-138: conj(h) * d / S
        dre[d] += (hre * dd.x + him * dd.y) * is;
        dim[d] += (hre * dd.y - him * dd.x) * is;
        hh[d] += (hre * hre + him * him) * is;
      }
    }
  }
#pragma unroll
  for (int d = 0; d < D; ++d) {
    out[d * kPartStride + 0] = dre[d];
    out[d * kPartStride + 1] = dim[d];
    out[d * kPartStride + 2] = hh[d];
  }
}

template <int D>
__global__ void __launch_bounds__(kPointsPerCta) k_plain_tf2(LaunchArgs a) {
  constexpr int CH = kChunkPlain;
  __shared__ double s_f[CH];
  __shared__ double2 s_d[D][CH];
  __shared__ double s_is[D][CH];
  const int64_t k0 = a.k_base + (int64_t)blockIdx.y * CH;
  for (int j = threadIdx.x; j < CH; j += blockDim.x) {
    const int64_t k = k0 + j;
    s_f[j] = a.freq[k];
#pragma unroll
    for (int d = 0; d < D; ++d) {
      s_d[d][j] = reinterpret_cast<const double2*>(a.strain[d])[k];
      s_is[d][j] = a.inv_psd[d][k];
    }
  }
  __syncthreads();
  const int64_t i = (int64_t)blockIdx.x * kPointsPerCta + threadIdx.x;
  if (i >= a.B) return;
  const PointRec& r = a.rec[i];
  double* out = a.part + (((int64_t)blockIdx.y * a.B + i) * D) * kPartStride;
  double dre[D], dim[D], hh[D], fp[D], fx[D], w2[D];
#pragma unroll
  for (int d = 0; d < D; ++d) {
    dre[d] = dim[d] = hh[d] = 0.0;
    fp[d] = r.fp[d];
    fx[d] = r.fx[d];
    w2[d] = 2.0 * kPi * r.dt[d];
  }
  if (r.valid) {
    double ak[8], lk[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      ak[k] = r.a[k];
      lk[k] = r.l[k];
    }
    const double pim = kPi * r.m_sec, amp0 = r.amp, ci = r.cos_i, f_isco = r.f_isco;
    const double pref = 3.0 / (128.0 * r.eta), cphase = -2.0 * r.phase - kPi / 4;
    const double pfac = (1.0 + ci * ci) / 2.0;
    for (int j = 0; j < CH; ++j) {
      const double f = s_f[j];
      if (f < a.fmin || f >= f_isco) continue;
      // the TaylorF2 model (oracle/taylorf2.py) evaluated in float64
      const double v = cbrt(pim * f);
      const double lnv = log(v);
      double s = 0.0, vk = 1.0;
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        s = s + (ak[k] + lk[k] * lnv) * vk;
        vk = vk * v;
      }
      const double v5 = v * v * v * v * v;
      const double psi = cphase + pref * s / v5;
      const double amp = amp0 * pow(f, -7.0 / 6.0);
      double sp, cp;
      sincos(psi, &sp, &cp);  // exp(-i psi) = cp - i sp
      const double ere = amp * cp, eim = -amp * sp;
      // h_+ = pfac * e, h_x = -i ci * e
      const double hpre = pfac * ere, hpim = pfac * eim;
      const double hxre = ci * eim, hxim = -ci * ere;
#pragma unroll
      for (int d = 0; d < D; ++d) {
        const double is = s_is[d][j];
        if (is == 0.0) continue;
        const double sre = hpre * fp[d] + hxre * fx[d];
        const double sim = hpim * fp[d] + hxim * fx[d];
        double sn, cs;
        sincos(w2[d] * f, &sn, &cs);
        const double hre = sre * cs + sim * sn;
        const double him = sim * cs - sre * sn;
        const double2 dd = s_d[d][j];
        dre[d] += (hre * dd.x + him * dd.y) * is;
        dim[d] += (hre * dd.y - him * dd.x) * is;
        hh[d] += (hre * hre + him * him) * is;
      }
    }
  }
#pragma unroll
  for (int d = 0; d < D; ++d) {
    out[d * kPartStride + 0] = dre[d];
    out[d * kPartStride + 1] = dim[d];
    out[d * kPartStride + 2] = hh[d];
  }
}

// ---------------------------------------------------------------------------
// mixed-precision kernels
// ---------------------------------------------------------------------------
// Phase of bin k in cycles from the 0.64 fixed-point rate x: the top 32 bits
// of k * x mod 2^64, as a signed fraction of a cycle in [-1/2, 1/2).
__device__ __forceinline__ float fixed_phase_cycles(uint32_t k, uint32_t xlo, uint32_t xhi) {
  const uint32_t top = k * xhi + __umulhi(k, xlo);
  return __int2float_rn((int)top) * 2.3283064365386963e-10f;  // 2^-32
}

constexpr int kFlush = 64;  // bins summed in float32 before folding into float64

// TaylorF2, mixed precision.  Shared memory per chunk: the float-float phase
// basis (64 B/bin) and each detector's weights f^(-7/6) d / S (8 B/bin/det),
// brought in by 1-D bulk async copies completed on one mbarrier.
template <int D>
__global__ void __launch_bounds__(kPointsPerCta) k_mixed_tf2(LaunchArgs a) {
  constexpr int CH = kChunkMixed;
  extern __shared__ __align__(128) unsigned char smem[];
  float2* s_basis = reinterpret_cast<float2*>(smem);                     // [CH][8]
  float2* s_w = reinterpret_cast<float2*>(smem + CH * kNumBasis * 8);   // [D][CH]
  __shared__ uint64_t bar;
  __shared__ int s_any;
  const int64_t k0 = a.k_base + (int64_t)blockIdx.y * CH;
  const int64_t i = (int64_t)blockIdx.x * kPointsPerCta + threadIdx.x;
  const bool have = i < a.B;
  int64_t ks = 0, ke = 0;
  int valid = 0;
  if (have) {
    valid = a.rec[i].valid;
    ks = a.rec[i].k_start;
    ke = a.rec[i].k_end;
  }
  const int64_t jb = max((int64_t)0, ks - k0);
  const int64_t je = min((int64_t)CH, ke - k0);
  const bool work = have && valid && jb < je;
  if (threadIdx.x == 0) s_any = 0;
  __syncthreads();
  if (work) s_any = 1;
  __syncthreads();
  double tre[D], tim[D];
#pragma unroll
  for (int d = 0; d < D; ++d) tre[d] = tim[d] = 0.0;
  if (s_any) {
    if (threadIdx.x == 0) {
      mbar_init(&bar, 1);
      mbar_fence_init();
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      const uint32_t bytes_basis = CH * kNumBasis * 8;
      const uint32_t bytes_w = CH * 8;
      mbar_expect_tx(&bar, bytes_basis + D * bytes_w);
      bulk_g2s(s_basis, a.basis + k0 * kNumBasis, bytes_basis, &bar);
#pragma unroll
      for (int d = 0; d < D; ++d) bulk_g2s(s_w + d * CH, a.w[d] + k0, bytes_w, &bar);
    }
    const bool arrived = mbar_wait_bounded(&bar, 0, a.status, kWaitLimit);
    if (arrived && work) {
      const PointRec& r = a.rec[i];
      float ch[kNumBasis + 1], cl[kNumBasis + 1];
#pragma unroll
      for (int b = 0; b <= kNumBasis; ++b) {
        ch[b] = r.c_hi[b];
        cl[b] = r.c_lo[b];
      }
      uint32_t xl[D], xh[D];
#pragma unroll
      for (int d = 0; d < D; ++d) {
        xl[d] = r.xfix[d][0];
        xh[d] = r.xfix[d][1];
      }
      for (int64_t jf = jb; jf < je; jf += kFlush) {
        const int jend = (int)min(je, jf + kFlush);
        float are[D], aim[D];
#pragma unroll
        for (int d = 0; d < D; ++d) are[d] = aim[d] = 0.f;
        for (int j = (int)jf; j < jend; ++j) {
          const float4* bp = reinterpret_cast<const float4*>(s_basis + j * kNumBasis);
          float s_hi = ch[kNumBasis], s_lo = cl[kNumBasis];
#pragma unroll
          for (int q = 0; q < kNumBasis / 2; ++q) {
            const float4 v = bp[q];
            ff_mac(s_hi, s_lo, ch[2 * q], cl[2 * q], v.x, v.y);
            ff_mac(s_hi, s_lo, ch[2 * q + 1], cl[2 * q + 1], v.z, v.w);
          }
          const float base = __fadd_rn(__fsub_rn(s_hi, rintf(s_hi)), s_lo);
          const uint32_t k = (uint32_t)(k0 + j);
#pragma unroll
          for (int d = 0; d < D; ++d) {
            float ph = base + fixed_phase_cycles(k, xl[d], xh[d]);
            ph -= rintf(ph);
            float sn, cs;
            __sincosf(ph * 6.283185307179586f, &sn, &cs);
            const float2 w = s_w[d * CH + j];
            are[d] = __fmaf_rn(w.x, cs, __fmaf_rn(-w.y, sn, are[d]));
            aim[d] = __fmaf_rn(w.x, sn, __fmaf_rn(w.y, cs, aim[d]));
          }
        }
#pragma unroll
        for (int d = 0; d < D; ++d) {
          tre[d] += are[d];
          tim[d] += aim[d];
        }
      }
    }
  }
  if (have) {
    double* out = a.part + (((int64_t)blockIdx.y * a.B + i) * D) * kPartStride;
#pragma unroll
    for (int d = 0; d < D; ++d) {
      out[d * kPartStride + 0] = tre[d];
      out[d * kPartStride + 1] = tim[d];
    }
  }
}

// Sine-Gaussian, mixed precision.  Shared memory per chunk: float32
// frequencies, each detector's weights d / S and 1 / S (scaled).
template <int D>
__global__ void __launch_bounds__(kPointsPerCta) k_mixed_sg(LaunchArgs a) {
  constexpr int CH = kChunkMixed;
  __shared__ __align__(16) float s_f[CH];
  __shared__ __align__(16) float2 s_w[D][CH];
  __shared__ __align__(16) float s_v[D][CH];
  __shared__ uint64_t bar;
  const int64_t k0 = a.k_base + (int64_t)blockIdx.y * CH;
  const int64_t i = (int64_t)blockIdx.x * kPointsPerCta + threadIdx.x;
  const bool have = i < a.B;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    mbar_fence_init();
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    mbar_expect_tx(&bar, CH * 4 + D * CH * 12);
    bulk_g2s(s_f, a.freq_f + k0, CH * 4, &bar);
#pragma unroll
    for (int d = 0; d < D; ++d) {
      bulk_g2s(s_w[d], a.w[d] + k0, CH * 8, &bar);
      bulk_g2s(s_v[d], a.v[d] + k0, CH * 4, &bar);
    }
  }
  const bool arrived = mbar_wait_bounded(&bar, 0, a.status, kWaitLimit);
  double t[D][6];
#pragma unroll
  for (int d = 0; d < D; ++d)
#pragma unroll
    for (int q = 0; q < 6; ++q) t[d][q] = 0.0;
  if (have && arrived && a.rec[i].valid) {
    const PointRec& r = a.rec[i];
    const float f0h = __double2float_rn(r.sg_f0);
    const float f0l = __double2float_rn(r.sg_f0 - (double)f0h);
    const float gah = __double2float_rn(r.sg_a);
    const float gal = __double2float_rn(r.sg_a - (double)gah);
    uint32_t xl[D], xh[D];
#pragma unroll
    for (int d = 0; d < D; ++d) {
      xl[d] = r.xfix[d][0];
      xh[d] = r.xfix[d][1];
    }
    for (int jf = 0; jf < CH; jf += kFlush) {
      float acc[D][6], cmp[D][6];
#pragma unroll
      for (int d = 0; d < D; ++d)
#pragma unroll
        for (int q = 0; q < 6; ++q) acc[d][q] = cmp[d][q] = 0.f;
      for (int j = jf; j < jf + kFlush; ++j) {
        const float f = s_f[j];
        const float g1 = gauss_ff(f, f0h, f0l, gah, gal, -1.0f);
        const float g2 = gauss_ff(f, f0h, f0l, gah, gal, 1.0f);
        const float hp = g1 + g2, hx = g1 - g2;
        const float hp2 = hp * hp, hx2 = hx * hx;
        const uint32_t k = (uint32_t)(k0 + j);
#pragma unroll
        for (int d = 0; d < D; ++d) {
          // The sine-Gaussian's phase is linear in k, so the error of the
          // hardware sin/cos approximation would repeat coherently from bin
          // to bin: use the accurate sincospi on the exact fraction.
          const float ph = fixed_phase_cycles(k, xl[d], xh[d]);
          float sn, cs;
          sincospif(2.0f * ph, &sn, &cs);
          const float2 w = s_w[d][j];
          const float ere = w.x * cs - w.y * sn, eim = w.x * sn + w.y * cs;
          const float vv = s_v[d][j];
          kahan_add(acc[d][0], cmp[d][0], hp * ere);
          kahan_add(acc[d][1], cmp[d][1], hp * eim);
          kahan_add(acc[d][2], cmp[d][2], hx * ere);
          kahan_add(acc[d][3], cmp[d][3], hx * eim);
          kahan_add(acc[d][4], cmp[d][4], hp2 * vv);
          kahan_add(acc[d][5], cmp[d][5], hx2 * vv);
        }
      }
#pragma unroll
      for (int d = 0; d < D; ++d)
#pragma unroll
        for (int q = 0; q < 6; ++q) t[d][q] += (double)acc[d][q] - (double)cmp[d][q];
    }
  }
  if (have) {
    double* out = a.part + (((int64_t)blockIdx.y * a.B + i) * D) * kPartStride;
#pragma unroll
    for (int d = 0; d < D; ++d)
#pragma unroll
      for (int q = 0; q < 6; ++q) out[d * kPartStride + q] = t[d][q];
  }
}

// ---------------------------------------------------------------------------
// finalize: fixed-order reduction over chunks, <d|h>, <h|h>, marginalisation
// ---------------------------------------------------------------------------
__device__ __forceinline__ double neg_huge() { return -1.7976931348623157e308; }  // nan_to_num(-inf)

__device__ void detector_totals(const LaunchArgs& a, int64_t i, const PointRec& r, double* dh_re, double* dh_im,
                                double* hh) {
  const double norm = 4.0 / a.duration;
  double sdr = 0.0, sdi = 0.0, shh = 0.0;
  for (int d = 0; d < a.n_det; ++d) {
    double p[kPartStride] = {0, 0, 0, 0, 0, 0};
    for (int64_t c = 0; c < a.n_chunks; ++c) {
      const double* q = a.part + ((c * a.B + i) * a.n_det + d) * kPartStride;
      const int nq = a.precision == GWL_PRECISION_FP64 ? 3 : (a.model == GWL_MODEL_SINEGAUSSIAN ? 6 : 2);
      for (int t = 0; t < nq; ++t) p[t] += q[t];
    }
    double dr, di, h;
    if (a.precision == GWL_PRECISION_FP64) {
      dr = norm * p[0];
      di = norm * p[1];
      h = norm * p[2];
    } else if (a.model == GWL_MODEL_SINEGAUSSIAN) {
      // conj(h) = (Fp P hp + i Fx X hx) e^{+i theta}; sums S1 = sum hp e w, S2 = sum hx e w
      const double P = r.amp, X = r.amp2, ws = a.w_scale[d], vs = a.v_scale[d];
      const double A = r.fp[d] * P, C = r.fx[d] * X;
      dr = norm * ws * (A * p[0] - C * p[3]);
      di = norm * ws * (A * p[1] + C * p[2]);
      h = norm * vs * (A * A * p[4] + C * C * p[5]);
    } else {
      // conj(h_det) = A0 f^(-7/6) conj(Q) e^{+i Phi},  Q = Fp (1 + c^2)/2 - i Fx c
      const double ci = r.cos_i;
      const double qr = r.fp[d] * (1.0 + ci * ci) / 2.0, qi = -r.fx[d] * ci;
      const double s = norm * a.w_scale[d] * r.amp;
      // (qr - i qi) * (p0 + i p1)
      dr = s * (qr * p[0] + qi * p[1]);
      di = s * (qr * p[1] - qi * p[0]);
      const int64_t k1 = min(r.k_end, a.n_bins), k0 = min(r.k_start, k1);
      const double* pre = a.hh_prefix[d];
      h = norm * r.amp * r.amp * (qr * qr + qi * qi) * (pre[k1] - pre[k0]);
    }
    sdr += dr;
    sdi += di;
    shh += h;
  }
  *dh_re = sdr;
  *dh_im = sdi;
  *hh = shh;
}

__device__ double distance_marginalized(const LaunchArgs& a, double dh_re, double dh_im, double hh, double dist) {
  // base.py:775-784, 879-885
  const double hh_ref = hh * dist * dist / (a.ref_dist * a.ref_dist);
  const double sr = dist / a.ref_dist;
  const double dr = dh_re * sr, di = dh_im * sr;
  const double x = a.phase_marg ? sqrt(dr * dr + di * di) : dr;
  return bicubic_eval(a.tx, a.nx, a.ty, a.ny, a.tc, a.bbox, x, hh_ref);
}

__global__ void k_finalize(LaunchArgs a) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.B) return;
  const PointRec& r = a.rec[i];
  double dr, di, hh;
  detector_totals(a, i, r, &dr, &di, &hh);
  if (a.dh_out) {
    a.dh_out[2 * i] = dr;
    a.dh_out[2 * i + 1] = di;
  }
  if (a.hh_out) a.hh_out[i] = hh;
  if (!a.out) return;
  double lnl;
  if (!r.valid) {
    lnl = neg_huge();
  } else if (a.dist_marg) {
    lnl = distance_marginalized(a, dr, di, hh, r.dist);
  } else if (a.phase_marg) {
    lnl = ln_i0(sqrt(dr * dr + di * di)) - hh / 2;  // base.py:786-792
  } else {
    lnl = dr - hh / 2;  // base.py:475
  }
  a.out[i] = lnl;
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
cudaError_t launch_prologue(const LaunchArgs& a, cudaStream_t s) {
  const int threads = 128;
  k_prologue<<<(unsigned)((a.B + threads - 1) / threads), threads, 0, s>>>(a);
  return cudaGetLastError();
}

#define GWL_DISPATCH_D(KERNEL, GRID, BLOCK, SMEM, STREAM, ARGS)          \
  switch ((ARGS).n_det) {                                               \
    case 1: KERNEL<1><<<GRID, BLOCK, SMEM, STREAM>>>(ARGS); break;      \
    case 2: KERNEL<2><<<GRID, BLOCK, SMEM, STREAM>>>(ARGS); break;      \
    case 3: KERNEL<3><<<GRID, BLOCK, SMEM, STREAM>>>(ARGS); break;      \
    default: KERNEL<4><<<GRID, BLOCK, SMEM, STREAM>>>(ARGS); break;     \
  }

cudaError_t launch_plain(const LaunchArgs& a, cudaStream_t s) {
  dim3 grid((unsigned)((a.B + kPointsPerCta - 1) / kPointsPerCta), (unsigned)a.n_chunks);
  if (a.model == GWL_MODEL_SINEGAUSSIAN) {
    GWL_DISPATCH_D(k_plain_sg, grid, kPointsPerCta, 0, s, a);
  } else {
    GWL_DISPATCH_D(k_plain_tf2, grid, kPointsPerCta, 0, s, a);
  }
  return cudaGetLastError();
}

template <int D>
static cudaError_t set_mixed_smem() {
  const int bytes = kChunkMixed * kNumBasis * 8 + D * kChunkMixed * 8;
  return cudaFuncSetAttribute(k_mixed_tf2<D>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}

cudaError_t launch_mixed(const LaunchArgs& a, cudaStream_t s) {
  dim3 grid((unsigned)((a.B + kPointsPerCta - 1) / kPointsPerCta), (unsigned)a.n_chunks);
  if (a.model == GWL_MODEL_SINEGAUSSIAN) {
    GWL_DISPATCH_D(k_mixed_sg, grid, kPointsPerCta, 0, s, a);
  } else {
    static bool configured = false;
    if (!configured) {
      cudaError_t e;
      if ((e = set_mixed_smem<1>()) != cudaSuccess) return e;
      if ((e = set_mixed_smem<2>()) != cudaSuccess) return e;
      if ((e = set_mixed_smem<3>()) != cudaSuccess) return e;
      if ((e = set_mixed_smem<4>()) != cudaSuccess) return e;
      configured = true;
    }
    const int smem = kChunkMixed * kNumBasis * 8 + a.n_det * kChunkMixed * 8;
    GWL_DISPATCH_D(k_mixed_tf2, grid, kPointsPerCta, smem, s, a);
  }
  return cudaGetLastError();
}

cudaError_t launch_finalize(const LaunchArgs& a, cudaStream_t s) {
  const int threads = 128;
  k_finalize<<<(unsigned)((a.B + threads - 1) / threads), threads, 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace gwl
