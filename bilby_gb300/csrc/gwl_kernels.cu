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
#include "gwl_marg_common.cuh"
#include "gwl_math.cuh"
#include "gwl_phase.cuh"

namespace gwl {

__device__ __forceinline__ double par(const LaunchArgs& a, int slot, int64_t i) {
  return a.params[(int64_t)slot * a.B + i];
}

// ---------------------------------------------------------------------------
// point ordering: bucket of a point = the chunk that holds its band end;
// points marked for the accurate kernel take the upper half of the keys, so
// that (buckets in descending order) they fill the first slots
// ---------------------------------------------------------------------------
__device__ __forceinline__ int order_key(const LaunchArgs& a, const PointRec& r) {
  if (a.model == GWL_MODEL_SINEGAUSSIAN) {
    // sine-Gaussian: the bin of the centre frequency, so that the points of a
    // warp walk their Gaussians (k_mixed_sg) over runs of nearly equal length
    if (!r.valid) return 0;
    const double kp = floor((r.sg_f0 - a.freq[a.k_base]) / a.step);
    const double n = (double)(a.n_chunks * a.chunk);
    return (int)((int64_t)fmin(fmax(kp, 0.0), n) >> a.order_shift);
  }
  if (!r.valid || r.k_end <= r.k_start) return 0;
  int64_t c = (r.k_end - a.k_base + a.chunk - 1) / a.chunk;
  c = c < 0 ? 0 : (c > a.n_chunks ? a.n_chunks : c);
  return (int)(c >> a.order_shift) + (r.refine ? a.order_half : 0);
}

// ---------------------------------------------------------------------------
// prologue: per-point float64 set-up (sky frame, antenna, delays, model scalars)
// ---------------------------------------------------------------------------
__device__ __noinline__ void prologue_point(const LaunchArgs& a, int64_t i) {
  PointRec r;
  memset(&r, 0, sizeof(r));
  const double ra = par(a, GWL_P_RA, i), dec = par(a, GWL_P_DEC, i), psi = par(a, GWL_P_PSI, i);
  double tgeo = par(a, GWL_P_GEOCENT_TIME, i);
  r.jitter = a.time_marg && a.jitter ? par(a, GWL_P_TIME_JITTER, i) : 0.0;
  // base.py:427-428: the jitter is added to geocent_time before projection.
  tgeo = tgeo + r.jitter;
  const double gmst = pymod(gmst_radians(tgeo), kTwoPi);
  bool ok = isfinite(ra) && isfinite(dec) && isfinite(psi) && isfinite(tgeo);
  const SkyTrig sky = sky_trig(ra, dec, psi, gmst);
  // an interferometer reference time (multiband.py:724-725, interferometer.py:333-336)
  // fixes the time of the antenna patterns; the delay stays at geocent_time
  const SkyTrig sky_ant =
      a.antenna_fixed ? sky_trig(ra, dec, psi, pymod(gmst_radians(a.antenna_time), kTwoPi)) : sky;
  for (int d = 0; d < a.n_det; ++d) {
    double fp, fx, delay;
    antenna_and_delay(a.det[d].tensor, a.det[d].vertex, sky, &fp, &fx, &delay);
    double delay_ref = delay;
    if (a.antenna_fixed) antenna_and_delay(a.det[d].tensor, a.det[d].vertex, sky_ant, &fp, &fx, &delay_ref);
    r.fp[d] = fp;
    r.fx[d] = fx;
    // interferometer.py:355-358: subtract the two GPS times first, then add the delay.
    const double dt_geocent = tgeo - a.det[d].start_time;
    // ROQ with time marginalisation: the delay at the antenna time alone (roq.py:529-541)
    r.dt[d] = a.roq_tm ? delay_ref : dt_geocent + delay;
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
    r.dist = dl;
    // Mc^(5/6) = eta^(1/2) M^(5/6) and M^(5/6) = M (cbrt(pi) / u)^(1/2) with u = (pi M)^(1/3)
    const double u = cbrt(kPi * r.m_sec);
    const double mc56 = sqrt(r.eta) * r.m_sec * sqrt(1.4645918875615231 / u);
    // sqrt(5/24) pi^(-2/3)
    r.amp = 0.45643546458763845 * 0.46619407703541166 * mc56 * kSpeedOfLight / (dl * 1e6 * kPcSI);
    r.cos_i = cos(theta_jn);
    r.phase = phase;
    // Re <d|h>_d = |Q_d| Re sum w e^{i (phase_k + alpha_d)}, alpha_d = arg(conj(Q_d)): the real-part
    // kernel carries alpha_d as a constant phase offset of detector d
    for (int d = 0; d < a.n_det; ++d) {
      const double qr = r.fp[d] * (1.0 + r.cos_i * r.cos_i) / 2.0, qi = -r.fx[d] * r.cos_i;
      r.qabs[d] = hypot(qr, qi);
      uint64_t u = 0;
      if (!a.cplx) {
        const double x = atan2(-qi, qr) / kTwoPi;
        double scaled = ldexp(x - floor(x), 64);
        if (!(scaled < 18446744073709551616.0)) scaled = 0.0;
        u = (uint64_t)scaled;
      }
      r.qfix[d][0] = (uint32_t)(u & 0xffffffffull);
      r.qfix[d][1] = (uint32_t)(u >> 32);
    }
    taylorf2_coefficients(m1, m2, chi1, chi2, r.a, r.l);
    ok = ok && m1 > 0 && m2 > 0 && dl > 0 && isfinite(r.amp) && isfinite(phase) && isfinite(chi1) &&
         isfinite(chi2);
    // band [k_start, k_end): f >= minimum_frequency and f < f_isco; k_end is
    // the first k with freq[k] >= f_isco: guessed from the uniform grid and
    // corrected against the frequency array (binary search if that fails)
    int64_t ke = (int64_t)fmin(fmax(ceil(r.f_isco / a.step), 0.0), (double)a.n_bins);
    for (int q = 0; q < 4 && ke > 0 && a.freq[ke - 1] >= r.f_isco; ++q) --ke;
    for (int q = 0; q < 4 && ke < a.n_bins && a.freq[ke] < r.f_isco; ++q) ++ke;
    if ((ke > 0 && a.freq[ke - 1] >= r.f_isco) || (ke < a.n_bins && a.freq[ke] < r.f_isco)) {
      int64_t lo = 0, hi = a.n_bins;
      while (lo < hi) {
        const int64_t mid = (lo + hi) / 2;
        if (a.freq[mid] >= r.f_isco) hi = mid; else lo = mid + 1;
      }
      ke = lo;
    }
    r.k_end = ke;
    r.k_start = a.k_fmin;
    // Psi / (2 pi) = sum_b c_b phi_b(f) + c_const with v = u f^(1/3), u = (pi M)^(1/3)
    const double P = 3.0 / (128.0 * r.eta) / kTwoPi;
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
  if (a.rf_tol > 0 && a.rf_count && r.valid && a.model == GWL_MODEL_TAYLORF2) {
    // error bound of the fast mixed-precision sums (kRefineL2): norms of the
    // per-bin terms |<d|h>_k| = 4/T A0 |Q_d| f^(-7/6) |d_k| / S_k over the band
    const int64_t k1 = min(r.k_end, a.n_bins), k0 = min(r.k_start, k1);
    double l2 = 0.0, l1 = 0.0;
    for (int d = 0; d < a.n_det; ++d) {
      const double s = 4.0 / a.duration * a.w_scale[d] * r.amp * r.qabs[d];
      l2 += s * s * (a.rf_p2[d][k1] - a.rf_p2[d][k0]);
      l1 += s * (a.rf_p1[d][k1] - a.rf_p1[d][k0]);
    }
    // (times the distance slope bound: the lnL's change per unit <d|h>)
    const double slope = a.dist_slope > 1.0 ? a.dist_slope : 1.0;
    if (slope * (kRefineL2 * sqrt(fmax(l2, 0.0)) + kRefineL1 * l1) > a.rf_tol) {
      r.refine = 1;
      atomicAdd(a.rf_count, 1);
      if (a.rf_total) atomicAdd(a.rf_total, 1);
    }
  }
  if (a.time_marg && a.precision == GWL_PRECISION_MIXED && a.n_fft > 0 && !a.relbin && !a.mb_tm && !a.roq) {
    // the mixed full-grid time-marginalised kernel's per-point scalars:
    // integrand coefficients, the TaylorF2 <h|h> and the exact sample window
    const double norm = 4.0 / a.duration;
    double hh = 0.0;
    for (int d = 0; d < a.n_det; ++d) {
      if (a.model == GWL_MODEL_TAYLORF2) {
        const double ci = r.cos_i;
        const double s = norm * r.amp * a.w_scale[d];
        r.tm_coef[2 * d] = (float)(s * r.fp[d] * (1.0 + ci * ci) / 2.0);
        r.tm_coef[2 * d + 1] = (float)(-s * r.fx[d] * ci);
        const double qr = r.fp[d] * (1.0 + ci * ci) / 2.0, qi = -r.fx[d] * ci;
        const int64_t k1 = min(r.k_end, a.n_bins), k0 = min(r.k_start, k1);
        hh += norm * r.amp * r.amp * (qr * qr + qi * qi) * (a.hh_prefix[d][k1] - a.hh_prefix[d][k0]);
      } else {
        r.tm_coef[2 * d] = (float)(norm * a.w_scale[d] * r.fp[d] * r.amp);
        r.tm_coef[2 * d + 1] = (float)(norm * a.w_scale[d] * r.fx[d] * r.amp2);
      }
    }
    r.tm_hh = hh;
    if (a.model == GWL_MODEL_TAYLORF2 && a.dist_marg) {
      // the distance spline's row at this point's <h|h> (base.py:775-784)
      const double sr = r.dist * a.inv_ref_dist;
      const SplineRowF row = bicubic_row_f(a.ty_f, a.ny, a.bbox, (float)(hh * sr * sr));
      r.tm_row_ly = row.Ly;
      r.tm_row_in = row.inside;
      for (int q = 0; q < 4; ++q) r.tm_row_hy[q] = row.hy[q];
    }
    // samples j with t_j = start + (j + 1) T / L + jitter inside [t_min, t_max]
    // (base.py:1027-1035), tested as the float64 kernel tests them; t_j
    // increases with j
    const int64_t L = a.n_fft;
    int64_t lo = 0, hi = L;
    while (lo < hi) {
      const int64_t mid = (lo + hi) / 2;
      if (tm_sample_time(a, mid, L, a.tm_step, r.jitter) >= a.t_min) hi = mid; else lo = mid + 1;
    }
    int64_t lo2 = lo, hi2 = L;
    while (lo2 < hi2) {
      const int64_t mid = (lo2 + hi2) / 2;
      if (tm_sample_time(a, mid, L, a.tm_step, r.jitter) <= a.t_max) lo2 = mid + 1; else hi2 = mid;
    }
    r.tm_j0 = lo;
    r.tm_j1 = lo2 - 1;
  }
  a.rec[i] = r;
  if (a.order_hist) atomicAdd(&a.order_hist[order_key(a, r)], 1);
}

__global__ void k_prologue(LaunchArgs a) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.B) return;
  prologue_point(a, i);
}

// Counts per bucket -> first slot of each bucket, buckets in descending order
// (longest bands first).  One CTA of kOrderThreads threads per analysis.
constexpr int kOrderThreads = 256;

__device__ void order_scan(const LaunchArgs& a) {
  __shared__ int s_part[kOrderThreads];
  const int n = a.order_keys, t = threadIdx.x;
  const int per = (n + kOrderThreads - 1) / kOrderThreads;
  int32_t* h = a.order_hist;
  int local = 0;
  for (int q = 0; q < per; ++q) {
    const int p = t * per + q;
    if (p < n) local += h[n - 1 - p];
  }
  s_part[t] = local;
  __syncthreads();
  for (int off = 1; off < kOrderThreads; off <<= 1) {
    const int v = t >= off ? s_part[t - off] : 0;
    __syncthreads();
    s_part[t] += v;
    __syncthreads();
  }
  int run = s_part[t] - local;
  for (int q = 0; q < per; ++q) {
    const int p = t * per + q;
    if (p < n) {
      const int key = n - 1 - p;
      const int c = h[key];
      h[key] = run;
      run += c;
    }
  }
}

// Slot of point i within its bucket (any order inside a bucket: the result of
// a point does not depend on the slot it is evaluated in).
__device__ __forceinline__ void order_scatter(const LaunchArgs& a, int64_t i) {
  const int key = order_key(a, a.rec[i]);
  const int pos = a.order_hist[key] + atomicAdd(&a.order_hist[a.order_keys + key], 1);
  if (pos >= 0 && pos < a.B) a.order[pos] = (int32_t)i;
  else atomicExch(a.status, kDevStatusBadInput);
}

__global__ void __launch_bounds__(kOrderThreads) k_order_scan(LaunchArgs a) { order_scan(a); }

__global__ void k_order_scatter(LaunchArgs a) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < a.B) order_scatter(a, i);
}

// ---------------------------------------------------------------------------
// plain float64 kernels
// ---------------------------------------------------------------------------
// (c + i s) *= (rc + i rs): one bin of a uniform-grid rotation.  Over a
// chunk of kChunkPlain bins its rounding error stays near 1e-13 rad.
__device__ __forceinline__ void rotate(double& c, double& s, double rc, double rs) {
  const double t = c * rc - s * rs;
  s = c * rs + s * rc;
  c = t;
}

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
    // e^{i w f} on the chunk's uniform grid by rotation from its first bin
    double zc[D], zs[D], rc[D], rs[D];
#pragma unroll
    for (int d = 0; d < D; ++d) {
      sincos(w2[d] * s_f[0], &zs[d], &zc[d]);
      sincos(w2[d] * a.step, &rs[d], &rc[d]);
    }
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
        const double sn = zs[d], cs = zc[d];  // exp(-i w f) = cs - i sn
        const double hre = sre * cs + sim * sn;
        const double him = sim * cs - sre * sn;
        const double2 dd = s_d[d][j];
        // utils.py:118-138: conj(h) * d / S
        dre[d] += (hre * dd.x + him * dd.y) * is;
        dim[d] += (hre * dd.y - him * dd.x) * is;
        hh[d] += (hre * hre + him * him) * is;
      }
#pragma unroll
      for (int d = 0; d < D; ++d) rotate(zc[d], zs[d], rc[d], rs[d]);
    }
  }
#pragma unroll
  for (int d = 0; d < D; ++d) {
    double* out = a.part + (((int64_t)blockIdx.y * D + d) * kPartStride) * a.B + i;
    out[0 * a.B] = dre[d];
    out[1 * a.B] = dim[d];
    out[2 * a.B] = hh[d];
  }
}

// TaylorF2, float64.  Per bin: v = u f^(1/3), ln v = ln u + ln(f) / 3 and
// the f^(-5/3), f^(-7/6) factors from the per-analysis table, the 3.5PN phase
// by Horner's rule, one sincos, and each detector's time shift e^{-2 pi i f dt}
// by rotation on the chunk's uniform grid.  <h|h> comes from the analysis's
// prefix sums of f^(-7/3) / S (finalize), so only <d|h> is summed here.
template <int D>
__global__ void __launch_bounds__(kPointsPerCta) k_plain_tf2(LaunchArgs a) {
  constexpr int CH = kChunkPlain;
  __shared__ double s_f[CH];
  __shared__ double4 s_t[CH];
  __shared__ double2 s_d[D][CH];
  __shared__ double s_is[D][CH];
  const int64_t k0 = a.k_base + (int64_t)blockIdx.y * CH;
  for (int j = threadIdx.x; j < CH; j += blockDim.x) {
    const int64_t k = k0 + j;
    s_f[j] = a.freq[k];
    s_t[j] = a.ftab[k];
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
  double dre[D], dim[D], fp[D], fx[D];
#pragma unroll
  for (int d = 0; d < D; ++d) {
    dre[d] = dim[d] = 0.0;
    fp[d] = r.fp[d];
    fx[d] = r.fx[d];
  }
  if (r.valid && k0 < r.k_end && k0 + CH > r.k_start) {
    double ak[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) ak[k] = r.a[k];
    const double l5 = r.l[5], l6 = r.l[6];
    const double u = cbrt(kPi * r.m_sec), lnu = log(u);
    const double amp0 = r.amp, ci = r.cos_i, f_isco = r.f_isco;
    const double pu5 = 3.0 / (128.0 * r.eta) / (u * u * u * u * u), cphase = -2.0 * r.phase - kPi / 4;
    const double pfac = (1.0 + ci * ci) / 2.0;
    double zc[D], zs[D], rc[D], rs[D];
#pragma unroll
    for (int d = 0; d < D; ++d) {
      const double w2 = 2.0 * kPi * r.dt[d];
      sincos(w2 * s_f[0], &zs[d], &zc[d]);
      sincos(w2 * a.step, &rs[d], &rc[d]);
    }
    for (int j = 0; j < CH; ++j) {
      const double f = s_f[j];
      if (f >= a.fmin && f < f_isco) {
        // the TaylorF2 model (oracle/taylorf2.py) evaluated in float64
        const double4 t = s_t[j];
        const double v = u * t.x;
        const double lnv = lnu + t.y;
        double s = ak[7];
#pragma unroll
        for (int k = 6; k >= 0; --k) s = s * v + ak[k];
        const double v5 = v * v * v * v * v;
        s = s + lnv * (l5 + l6 * v) * v5;
        const double psi = cphase + pu5 * s * t.z;
        const double amp = amp0 * t.w;
        double sp, cp;
        sincos(psi, &sp, &cp);  // exp(-i psi) = cp - i sp
        const double ere = amp * cp, eim = -amp * sp;
        // h_+ = pfac * e, h_x = -i ci * e
        const double hpre = pfac * ere, hpim = pfac * eim;
        const double hxre = ci * eim, hxim = -ci * ere;
#pragma unroll
        for (int d = 0; d < D; ++d) {
          const double is = s_is[d][j];
          const double sre = hpre * fp[d] + hxre * fx[d];
          const double sim = hpim * fp[d] + hxim * fx[d];
          const double sn = zs[d], cs = zc[d];  // exp(-i w f) = cs - i sn
          const double hre = sre * cs + sim * sn;
          const double him = sim * cs - sre * sn;
          const double2 dd = s_d[d][j];
          dre[d] += (hre * dd.x + him * dd.y) * is;
          dim[d] += (hre * dd.y - him * dd.x) * is;
        }
      }
#pragma unroll
      for (int d = 0; d < D; ++d) rotate(zc[d], zs[d], rc[d], rs[d]);
    }
  }
#pragma unroll
  for (int d = 0; d < D; ++d) {
    double* out = a.part + (((int64_t)blockIdx.y * D + d) * kPartStride) * a.B + i;
    out[0 * a.B] = dre[d];
    out[1 * a.B] = dim[d];
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

constexpr int kFlush = 64;  // bins summed in float32 before folding into float64 (sine-Gaussian)
constexpr int kFold = 8;    // bins summed in float32 before folding into float-float (direct TaylorF2 chunks)

// TaylorF2, mixed precision.
//
// Phase: about anchor bins k_a (every J bins, J from the Taylor-remainder
// bound below) the phase in cycles Phi(k_a + j) = sum_n A_n j^n is a
// polynomial of degree 4 to 6 whose coefficients A_n = sum_b c_b T_n,b(k_a)
// come from the per-analysis Taylor tables of the basis functions (orders
// 0..3 in float-float).  It is split into a quadratic part Q(j) = A_0 + A_1 j
// + A_2 j^2 plus detector 0's time shift, kept exactly in 0.64 fixed point
// (cycles modulo one), and the rest C(j) = sum_{n >= 3} A_n j^n, a small
// fraction of a cycle over the interval, evaluated in float32.  Q is stepped
// once per 8-bin block with wrapping 64-bit integer adds, which are exact:
// its value and first difference at the block start, step-8 forward
// differences.  Inside a block the phase of bin i is the 32-bit top word
// top(i) = top(Q) + i top(dQ) (truncation error below 8 units of 2^-32
// cycle) plus the float32 remainder C(i, 2) 2 A_2 + C(j) (radians).  The
// detector time shifts relative to detector 0 are exact 0.64 sequences
// stepped per block, and their 32-bit slope per bin is added inside it.
// The weight table of this kernel holds per bin pair {|w| even, |w| odd,
// tau even, tau odd}, tau the weight angle arg(w) at a block's first bin and
// the angle increment arg(w_k) - arg(w_{k-1}) elsewhere, so that each bin's
// 32-bit angle is one three-input add of the previous bin's.  Two bins run
// as one packed float pair (f32x2 multiply-adds); only the hardware cosine
// and the packed multiply-accumulate with the weights w = f^(-7/6) d / S are
// float32.  The even and odd bins' float32 partial sums (8 terms each) are
// folded every 16 bins into float-float accumulators.
//
// Work split (split-K): CTA (tile, g) holds 128 points and walks chunks
// g, g + G, ... of 512 bins; each chunk's weights come in by 1-D bulk async
// copies into a double-buffered shared-memory stage.  One partial sum per
// (g, detector, point) is written, point fastest.

// Accurate variant, for the points the prologue marks (LaunchArgs::rf_tol).
// The hardware cosine's error is a smooth function of the angle, so it adds up
// coherently where a template follows a loud signal in the data, and so do the
// roundings of float32 sums of 8 such terms.  Here cos and sin of 2 pi u 2^-32
// are float-float pairs hi + lo: the table entry at the nearest 1/kCosTable
// cycle (float-float of the float64 values) rotated by the remainder r,
// |r| <= pi / kCosTable, with cos r - 1 = -r^2/2 + r^4/24 and sin r = r - r^3/6
// (truncation below 3e-15); each term is added into the chunk's float-float
// sum by TwoSum.  What remains is rounding of single terms (the weight
// magnitude, the product), independent from bin to bin.
static_assert(kCosTable == 1024, "cos_sin_fixed splits the angle as 10 + 22 bits");

template <bool SIN>
__device__ __forceinline__ void cos_sin_fixed(const float4* tab, uint32_t u, float& ch, float& cl, float& sh,
                                              float& sl) {
  const uint32_t q = (u + (1u << 21)) >> 22;  // nearest table angle (q = kCosTable wraps to entry 0)
  const float r = __fmul_rn((float)(int32_t)(u - (q << 22)), 1.4629180792671596e-09f);  // |u - q 2^22| <= 2^21: exact
  const float4 t = tab[q & (kCosTable - 1)];
  const float z = __fmul_rn(r, r);
  const float cm1 = __fmul_rn(z, __fmaf_rn(z, 1.0f / 24.0f, -0.5f));
  const float sr = __fmul_rn(r, __fmaf_rn(z, -1.0f / 6.0f, 1.0f));
  ch = t.x;
  cl = __fadd_rn(t.y, __fmaf_rn(t.x, cm1, -__fmul_rn(t.z, sr)));
  if (SIN) {
    sh = t.z;
    sl = __fadd_rn(t.w, __fmaf_rn(t.z, cm1, __fmul_rn(t.x, sr)));
  }
}

// hi + lo += m (c_hi + c_lo)
__device__ __forceinline__ void acc_ff(float& hi, float& lo, float m, float c_hi, float c_lo) {
  two_sum_acc(hi, lo, __fmul_rn(m, c_hi));
  lo = __fmaf_rn(m, c_lo, lo);
}

// One 8-bin block of the anchored walk, two bins per packed pair.  top[d]:
// detector d's 32-bit phase at the block start without the weight angle (on
// return: at the block's last bin, with it); sl[d]: its slope per bin.  wq:
// detector 0's four bin pairs of the block in the stage (detector d is
// kChunkMixed / 2 pairs further per detector).  jj: (j, j + 1) of the first
// pair relative to the anchor (advanced by 8).  A3, A4: the cubic and quartic
// Taylor coefficients in radians (both lanes equal), a5, a6 the quintic and
// sextic ones (zero below degree 5; HI blocks only), a2: the second
// difference of the quadratic part, whose local remainder is C(i, 2) a2.
// MASK: bins outside [lo, hi) contribute nothing (band edges).
template <int D, bool CPLX, bool HI, bool MASK>
__device__ __forceinline__ void tf2_block(uint32_t* top, const uint32_t* sl, const uint4* wq, float2& jj,
                                          float2 A3, float2 A4, float a5, float a6, float a2, int lo, int hi,
                                          float2* acc, float2* acci) {
  const float2 cc = make_float2(1.4629180792671596e-09f, 1.4629180792671596e-09f);  // 2 pi 2^-32
  const float2 two = make_float2(2.f, 2.f);
#pragma unroll
  for (int p = 0; p < 4; ++p) {
    float2 t = HI ? fma2(fma2(make_float2(a6, a6), jj, make_float2(a5, a5)), jj, A4) : A4;
    t = fma2(t, jj, A3);
    float2 rq = mul2(mul2(t, mul2(jj, jj)), jj);
    // + C(i, 2) a2 for bins i = 2p, 2p + 1 (binomials 0 1 3 6 10 15 21 28 ...)
    if (p > 0) {
      rq.x = __fmaf_rn(a2, (float)((2 * p) * (2 * p - 1) / 2), rq.x);
      rq.y = __fmaf_rn(a2, (float)((2 * p + 1) * (2 * p) / 2), rq.y);
    }
    jj = add2(jj, two);
#pragma unroll
    for (int d = 0; d < D; ++d) {
      const uint4 q = wq[d * (kChunkMixed / 2) + p];
      const uint32_t ta = p == 0 ? top[d] + q.z : top[d] + sl[d] + q.z;
      const uint32_t tb = ta + sl[d] + q.w;
      top[d] = tb;
      const float2 ph = fma2(make_float2(__int2float_rn((int)ta), __int2float_rn((int)tb)), cc, rq);
      float2 mag = make_float2(__uint_as_float(q.x), __uint_as_float(q.y));
      if (MASK) {
        mag.x = (2 * p >= lo && 2 * p < hi) ? mag.x : 0.f;
        mag.y = (2 * p + 1 >= lo && 2 * p + 1 < hi) ? mag.y : 0.f;
      }
      if (CPLX) {
        float s0, c0, s1, c1;
        __sincosf(ph.x, &s0, &c0);
        __sincosf(ph.y, &s1, &c1);
        acc[d] = fma2(mag, make_float2(c0, c1), acc[d]);
        acci[d] = fma2(mag, make_float2(s0, s1), acci[d]);
      } else {
        acc[d] = fma2(mag, make_float2(__cosf(ph.x), __cosf(ph.y)), acc[d]);
      }
    }
  }
}

// A chunk where no anchor interval meets the Taylor bound: the phase of every
// bin in float-float from the per-bin basis table (sum_b c_b phi_b(f_k)),
// the time shift exact in 0.64 fixed point; the weights from the plain polar
// table in global memory.
template <int D, bool CPLX>
__device__ __forceinline__ void direct_chunk(const LaunchArgs& a, int64_t k0, int64_t ks, int jlast,
                                             const float* ch, const float* cl, const uint64_t* X, const uint64_t* Q,
                                             float* ahi, float* alo, float* bhi, float* blo) {
  for (int jb = 0; jb < jlast; jb += kFold) {
    float are[D], aim[D];
#pragma unroll
    for (int d = 0; d < D; ++d) are[d] = aim[d] = 0.f;
    const int je = min(jb + kFold, jlast);
    for (int j = jb; j < je; ++j) {
      const int64_t k = k0 + j;
      if (k < ks) continue;
      const float4* bp = reinterpret_cast<const float4*>(a.basis + k * kNumBasis);
      float s_hi = ch[kNumBasis], s_lo = cl[kNumBasis];
#pragma unroll
      for (int q = 0; q < kNumBasis / 2; ++q) {
        const float4 v = __ldg(bp + q);
        ff_mac(s_hi, s_lo, ch[2 * q], cl[2 * q], v.x, v.y);
        ff_mac(s_hi, s_lo, ch[2 * q + 1], cl[2 * q + 1], v.z, v.w);
      }
      const uint32_t bu = (uint32_t)((to_fixed(s_hi, s_lo) + 0x80000000ull) >> 32);
#pragma unroll
      for (int d = 0; d < D; ++d) {
        const uint2 wv = __ldg(a.wp[d] + k);
        const uint32_t top = bu + (uint32_t)(((uint64_t)k * X[d] + Q[d]) >> 32) + wv.y;
        const float ph = __fmul_rn(__int2float_rn((int)top), 1.4629180792671596e-09f);
        float sn, cs;
        __sincosf(ph, &sn, &cs);
        const float mag = __uint_as_float(wv.x);
        are[d] = __fmaf_rn(mag, cs, are[d]);
        if (CPLX) aim[d] = __fmaf_rn(mag, sn, aim[d]);
      }
    }
#pragma unroll
    for (int d = 0; d < D; ++d) {
      two_sum_acc(ahi[d], alo[d], are[d]);
      if (CPLX) two_sum_acc(bhi[d], blo[d], aim[d]);
    }
  }
}

// One work unit: the points of tile `tile` over the chunks g, g + G, ...
// `it_global` counts the chunks this CTA has consumed so far (all units): it
// selects the shared-memory stage and the mbarrier phase.  The first n_acc
// slots hold the points marked by the prologue (the ordering puts them
// first): the accurate kernel evaluates them, this one skips them.
template <int D, bool CPLX>
__device__ __noinline__ void tf2_unit(const LaunchArgs& a, int64_t tile, int64_t g, uint2* s_w, uint64_t* bar,
                         unsigned long long* s_kmax, int64_t& it_global, int64_t n_acc) {
  constexpr int CH = kChunkMixed;
  const int64_t slot = tile * kPointsPerCta + threadIdx.x;
  const int64_t i = slot < a.B && a.order ? (int64_t)a.order[slot] : slot;
  const int64_t G = a.n_groups;
  const bool have = slot < a.B && i >= 0 && i < a.B && slot >= n_acc;
  int64_t ks = 0, ke = 0;
  bool valid = false;
  if (have) {
    valid = a.rec[i].valid != 0;
    ks = a.rec[i].k_start;
    ke = a.rec[i].k_end;
  }
  if (threadIdx.x == 0) *s_kmax = 0ull;
  __syncthreads();
  if (have && valid && ke > ks) atomicMax(s_kmax, (unsigned long long)ke);
  __syncthreads();
  const int64_t kmax = (int64_t)*s_kmax;
  // chunks of this group that can contribute: k0 < kmax
  const int64_t c_end = min(a.n_chunks, (kmax - a.k_base + CH - 1) / CH);
  const int64_t nit = c_end > g ? (c_end - g + G - 1) / G : 0;

  // the point's record: basis coefficients, time shifts and offsets are read
  // from it where they are needed (anchor set-ups), not held in registers
  const PointRec* rp = have ? a.rec + i : a.rec;
  float c0 = 0.f;
  // constant phase offset of detector d (real-part kernel), read when needed
  const auto qoff = [&](int d) -> uint64_t {
    if (CPLX) return 0;
    return ((uint64_t)rp->qfix[d][1] << 32) | rp->qfix[d][0];
  };
  const auto xfix = [&](int d) -> uint64_t { return ((uint64_t)rp->xfix[d][1] << 32) | rp->xfix[d][0]; };
  if (have && valid) c0 = fabsf(rp->c_hi[0]);
  // float32 partial sums folded into float-float accumulators, over every
  // chunk of the unit (real part; imaginary part for the complex kernel)
  float ahi[D], alo[D], bhi[D], blo[D];
#pragma unroll
  for (int d = 0; d < D; ++d) ahi[d] = alo[d] = bhi[d] = blo[d] = 0.f;

  const uint32_t stage_bytes = D * CH * 8;
  const int64_t it0 = it_global;
  if (nit > 0 && threadIdx.x == 0) {
    const int s0 = (int)(it0 & 1);
    const int64_t k0 = a.k_base + g * CH;
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    mbar_expect_tx(&bar[s0], stage_bytes);
#pragma unroll
    for (int d = 0; d < D; ++d) bulk_g2s(s_w + s0 * D * CH + d * CH, a.wq[d] + k0 / 2, CH * 8, &bar[s0]);
  }
  int64_t done = 0;
  for (int64_t it = 0; it < nit; ++it) {
    const int64_t itg = it0 + it;
    const int s = (int)(itg & 1);
    const int64_t c = g + it * G;
    if (it + 1 < nit && threadIdx.x == 0) {
      // the other stage was released by the barrier at the end of the previous iteration
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      const int64_t k1 = a.k_base + (c + G) * CH;
      uint2* dst = s_w + (s ^ 1) * D * CH;
      mbar_expect_tx(&bar[s ^ 1], stage_bytes);
#pragma unroll
      for (int d = 0; d < D; ++d) bulk_g2s(dst + d * CH, a.wq[d] + k1 / 2, CH * 8, &bar[s ^ 1]);
    }
    const bool arrived = mbar_wait_bounded(&bar[s], (uint32_t)((itg >> 1) & 1), a.status, kWaitLimit);
    done = it + 1;
    if (!__syncthreads_and(arrived)) break;
    const uint2* w = s_w + s * D * CH;
    const int64_t k0 = a.k_base + c * CH;
    if (have && valid && k0 < ke && k0 + CH > ks) {
      // this point's own anchor interval for the chunk: the result of a
      // point never depends on the other points of the batch
      const int J = anchor_interval(c0 * __powf((float)k0 * (float)a.step, -5.0f / 3.0f),
                                    (float)max(k0, (int64_t)8));
      const int jlast = (int)min((int64_t)CH, ke - k0);
      if (J == 0) {
        float ch[kNumBasis + 1], cl[kNumBasis + 1];
#pragma unroll
        for (int b = 0; b <= kNumBasis; ++b) {
          ch[b] = rp->c_hi[b];
          cl[b] = rp->c_lo[b];
        }
        uint64_t X[D], Q[D];
#pragma unroll
        for (int d = 0; d < D; ++d) {
          X[d] = xfix(d);
          Q[d] = qoff(d);
        }
        direct_chunk<D, CPLX>(a, k0, ks, jlast, ch, cl, X, Q, ahi, alo, bhi, blo);
      } else {
        // detector 0's time shift and constant offset ride in the exact
        // quadratic part (a linear term: Q(j) += (k + j) X0 + q0); detector
        // d > 0 adds its shift relative to detector 0, R_d = X_d - X_0, as an
        // exact 0.64 sequence L_d stepped per block, whose top word (rounded)
        // starts the block and whose rounded top word r32 is its slope per bin
        // (error at most 4.5 * 2^-32 cycle).  The +2^31 offsets make the top
        // words of E0, F0 and L_d rounded rather than truncated.
        uint64_t R8[D], L64[D];
        uint32_t r32[D];
#pragma unroll
        for (int d = 0; d < D; ++d) {
          const uint64_t Rd = xfix(d) - xfix(0);
          r32[d] = (uint32_t)((Rd + 0x80000000ull) >> 32);
          R8[d] = Rd * 8ull;
          L64[d] = 0;
        }
        // E0, E1, E2: Q at the block start and its step-8 differences; F0, F1:
        // dQ = Q(j + 1) - Q(j) at the block start and its step-8 difference
        uint64_t E0 = 0, E1 = 0, E2 = 0, F0 = 0, F1 = 0;
        const float2 zero2 = make_float2(0.f, 0.f);
        float2 A3 = zero2, A4 = zero2, jj = zero2;
        float a5 = 0.f, a6 = 0.f, a2 = 0.f;
        bool hi_deg = false;
        float2 acc[D], acci[D];
#pragma unroll
        for (int d = 0; d < D; ++d) acc[d] = acci[d] = zero2;
        const uint4* w4 = reinterpret_cast<const uint4*>(w);
        for (int jb = 0; jb < jlast; jb += 8) {
          const int64_t k = k0 + jb;
          if ((jb & (J - 1)) == 0) {
            const int deg = anchor_degree(c0 * __powf((float)k * (float)a.step, -5.0f / 3.0f), (float)J / (float)k);
            AnchorTaylor t;
            anchor_taylor(a.anchors, k, rp->c_hi, rp->c_lo, t);
            const uint64_t q0 = qoff(0), X0 = xfix(0);
            // Q(j) = A0 + A1 j + A2 j^2: Delta_8 Q(0) = 8 A1 + 64 A2, Delta_8^2 Q = 128 A2,
            // dQ(0) = A1 + A2, Delta_8 dQ = 16 A2 (scalings by powers of two are exact)
            float eh = 8.f * t.h[1], el = 8.f * t.l[1];
            ff_add(eh, el, 64.f * t.h[2], 64.f * t.l[2]);
            float fh = t.h[1], fl = t.l[1];
            ff_add(fh, fl, t.h[2], t.l[2]);
            E0 = to_fixed(t.h[0], t.l[0]) + (uint64_t)k * X0 + q0 + 0x80000000ull;
            E1 = to_fixed(eh, el) + 8ull * X0;
            E2 = to_fixed(128.f * t.h[2], 128.f * t.l[2]);
            F0 = to_fixed(fh, fl) + X0 + 0x80000000ull;
            F1 = to_fixed(16.f * t.h[2], 16.f * t.l[2]);
#pragma unroll
            for (int d = 1; d < D; ++d) L64[d] = (uint64_t)k * (xfix(d) - X0) + (qoff(d) - q0) + 0x80000000ull;
            // C(j) = j^3 (A3 + j (A4 + j (A5 + j A6))) in radians, truncated at degree deg
            const float tp = 6.283185307179586f;
            const float a3 = __fmul_rn(__fadd_rn(t.h[3], t.l[3]), tp), a4 = __fmul_rn(t.f[0], tp);
            a5 = deg >= 5 ? __fmul_rn(t.f[1], tp) : 0.f;
            a6 = deg >= 6 ? __fmul_rn(t.f[2], tp) : 0.f;
            A3 = make_float2(a3, a3);
            A4 = make_float2(a4, a4);
            hi_deg = deg > 4;
            // second difference of Q in radians: the local quadratic remainder
            // Q(jb + i) - Q(jb) - i dQ(jb) = C(i, 2) 2 A2
            a2 = __fmul_rn(2.f * t.h[2], tp);
            jj = make_float2(0.f, 1.f);
          }
          uint32_t top[D], sl[D];
          const uint32_t e0 = (uint32_t)(E0 >> 32), f0 = (uint32_t)(F0 >> 32);
#pragma unroll
          for (int d = 0; d < D; ++d) {
            top[d] = d == 0 ? e0 : e0 + (uint32_t)(L64[d] >> 32);
            sl[d] = d == 0 ? f0 : f0 + r32[d];
          }
          const uint4* wq = w4 + (jb >> 1);
          if (jb + 8 <= jlast && k >= ks) {
            // a whole block inside the band
            if (hi_deg) {
              tf2_block<D, CPLX, true, false>(top, sl, wq, jj, A3, A4, a5, a6, a2, 0, 8, acc, acci);
            } else {
              tf2_block<D, CPLX, false, false>(top, sl, wq, jj, A3, A4, a5, a6, a2, 0, 8, acc, acci);
            }
          } else {
            const int lo = (int)max((int64_t)0, ks - k), hi = min(8, jlast - jb);
            tf2_block<D, CPLX, true, true>(top, sl, wq, jj, A3, A4, a5, a6, a2, lo, hi, acc, acci);
          }
          E0 += E1;
          E1 += E2;
          F0 += F1;
#pragma unroll
          for (int d = 1; d < D; ++d) L64[d] += R8[d];
          if (jb & 8) {
            // every 16 bins: the even and odd partial sums into float-float
#pragma unroll
            for (int d = 0; d < D; ++d) {
              two_sum_acc(ahi[d], alo[d], __fadd_rn(acc[d].x, acc[d].y));
              if (CPLX) two_sum_acc(bhi[d], blo[d], __fadd_rn(acci[d].x, acci[d].y));
              acc[d] = acci[d] = zero2;
            }
          }
        }
#pragma unroll
        for (int d = 0; d < D; ++d) {
          two_sum_acc(ahi[d], alo[d], __fadd_rn(acc[d].x, acc[d].y));
          if (CPLX) two_sum_acc(bhi[d], blo[d], __fadd_rn(acci[d].x, acci[d].y));
        }
      }
    }
    __syncthreads();
  }
  it_global = it0 + done;
  if (have) {
#pragma unroll
    for (int d = 0; d < D; ++d) {
      a.part[((g * D + d) * kPartStride + 0) * a.B + i] = (double)ahi[d] + (double)alo[d];
      if (CPLX) a.part[((g * D + d) * kPartStride + 1) * a.B + i] = (double)bhi[d] + (double)blo[d];
    }
  }
}

template <int D, bool CPLX>
__global__ void __launch_bounds__(kPointsPerCta, 5) k_mixed_tf2(LaunchArgs a) {
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ uint64_t bar[2];
  __shared__ unsigned long long s_kmax;
  if (threadIdx.x == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    mbar_fence_init();
  }
  __syncthreads();
  int64_t it_global = 0;
  const int64_t n_acc = a.rf_count ? *a.rf_count : 0;
  tf2_unit<D, CPLX>(a, blockIdx.x, blockIdx.y, reinterpret_cast<uint2*>(smem), bar, &s_kmax, it_global, n_acc);
}

__device__ __forceinline__ void load_cos_table(float4* tab, const float4* src) {
  for (int q = threadIdx.x; q < kCosTable; q += blockDim.x) tab[q] = src[q];
}

// Accurate variant: one (marked point, chunk group) unit per warp.  Lane l
// takes bins k0 + l + 32 j of each chunk g, g + G, ... of the group (the
// chunks the fast kernel's CTA g walks), within the point's band.  Every bin's
// phase is evaluated in float-float from the basis table, so the lanes are
// independent (no recurrence to carry) and a point's 512-bin chunk costs 16
// bins of latency; the angle is summed in 64-bit fixed point (phase, time
// shift, detector offset, weight angle) and rounded once to 0.32; cos / sin
// from cos_sin_fixed; each term added by TwoSum; the lanes' sums reduced in
// float64 in a fixed order.  Writes the group's partial sums of the point.
constexpr int kAccThreads = 256;

template <int D, bool CPLX>
__device__ void acc_unit(const LaunchArgs& a, int64_t i, int64_t g, const float4* tab) {
  const int lane = threadIdx.x & 31;
  const PointRec& r = a.rec[i];
  const int64_t ks = r.k_start, ke = r.k_end;
  float ch[kNumBasis + 1], cl[kNumBasis + 1];
#pragma unroll
  for (int b = 0; b <= kNumBasis; ++b) {
    ch[b] = r.c_hi[b];
    cl[b] = r.c_lo[b];
  }
  uint64_t X[D], Q[D];
#pragma unroll
  for (int d = 0; d < D; ++d) {
    X[d] = ((uint64_t)r.xfix[d][1] << 32) | r.xfix[d][0];
    Q[d] = CPLX ? 0ull : (((uint64_t)r.qfix[d][1] << 32) | r.qfix[d][0]);
  }
  float ahi[D], alo[D], bhi[D], blo[D];
#pragma unroll
  for (int d = 0; d < D; ++d) ahi[d] = alo[d] = bhi[d] = blo[d] = 0.f;
  for (int64_t c = g; c < a.n_chunks; c += a.n_groups) {
    const int64_t k0 = a.k_base + c * kChunkMixed;
    if (k0 >= ke) break;
    if (k0 + kChunkMixed <= ks) continue;
    for (int j = lane; j < kChunkMixed; j += 32) {
      const int64_t k = k0 + j;
      if (k < ks || k >= ke) continue;
      const float4* bp = reinterpret_cast<const float4*>(a.basis + k * kNumBasis);
      float s_hi = ch[kNumBasis], s_lo = cl[kNumBasis];
#pragma unroll
      for (int q = 0; q < kNumBasis / 2; ++q) {
        const float4 v = __ldg(bp + q);
        ff_mac(s_hi, s_lo, ch[2 * q], cl[2 * q], v.x, v.y);
        ff_mac(s_hi, s_lo, ch[2 * q + 1], cl[2 * q + 1], v.z, v.w);
      }
      const uint64_t base = to_fixed(s_hi, s_lo);
#pragma unroll
      for (int d = 0; d < D; ++d) {
        const uint2 wv = __ldg(a.wp[d] + k);
        const uint64_t full = base + (uint64_t)k * X[d] + Q[d] + ((uint64_t)wv.y << 32);
        float c_h, c_l, s_h, s_l;
        cos_sin_fixed<CPLX>(tab, (uint32_t)((full + 0x80000000ull) >> 32), c_h, c_l, s_h, s_l);
        const float mag = __uint_as_float(wv.x);
        acc_ff(ahi[d], alo[d], mag, c_h, c_l);
        if (CPLX) acc_ff(bhi[d], blo[d], mag, s_h, s_l);
      }
    }
  }
#pragma unroll
  for (int d = 0; d < D; ++d) {
    double re = (double)ahi[d] + (double)alo[d];
    double im = CPLX ? (double)bhi[d] + (double)blo[d] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      re += __shfl_down_sync(0xffffffffu, re, o);
      if (CPLX) im += __shfl_down_sync(0xffffffffu, im, o);
    }
    if (lane == 0) {
      a.part[((g * D + d) * kPartStride + 0) * a.B + i] = re;
      if (CPLX) a.part[((g * D + d) * kPartStride + 1) * a.B + i] = im;
    }
  }
}

// The marked points (first rf_count slots of the ordering), all their groups;
// the count is read on the device, so the launch shape does not depend on it.
template <int D, bool CPLX>
__global__ void __launch_bounds__(kAccThreads) k_mixed_tf2_acc(LaunchArgs a) {
  __shared__ float4 tab[kCosTable];
  const int wpc = kAccThreads / 32;
  const int64_t units = (int64_t)*a.rf_count * a.n_groups;
  if ((int64_t)blockIdx.x * wpc >= units) return;
  load_cos_table(tab, a.cos_tab);
  __syncthreads();
  const int64_t nw = (int64_t)gridDim.x * wpc;
  for (int64_t u = (int64_t)blockIdx.x * wpc + (threadIdx.x >> 5); u < units; u += nw)
    acc_unit<D, CPLX>(a, a.order[u / a.n_groups], u % a.n_groups, tab);
}

// Sine-Gaussian, mixed precision (bilby/gw/source.py:1197-1207 projected as
// in interferometer.py:341-362, summed as in gw/utils.py:118-138).
//
// Per detector d the projection is conj(h_d) = M_d (a_d hp + i c_d hx) e^{+i theta}
// with hp = g1 + g2, hx = g1 - g2, g1,2 = exp(-pi^2 tau^2 (f -+ f0)^2),
// M_d = |(Fp P, Fx X)| and (a_d, c_d) = (Fp P, Fx X) / M_d.  Four partial sums:
//   0, 1: Re, Im of sum (a hp + i c hx) e^{i theta} w      (float32, Kahan)
//   2:    sum (a^2 hp^2 + c^2 hx^2) v                      (float-float)
//   3:    sum (a^2 hp^2 + c^2 hx^2) |w|^2                  (float32: error norm)
// The 0.32 fixed-point phase of bin k is exact; its float32 rounding is undone
// to first order (see the loop), so the phase contributes no error.
// Points are taken in the order of their centre frequencies (order_key), so
// that the threads of a warp walk runs of nearly equal lengths.
// <h|h> is float-float throughout: the Gaussians come from the float-float
// multiplicative recurrence g(k + s) = g(k) r(k), r(k + s) = r(k) c with
// c = exp(-2 A df^2) (A = pi^2 tau^2, s = +-1), walked away from the peak so
// that g only shrinks, started from float64 values at the first bin of each
// walk (each float-float product errs by about 2^-48, so after n steps the
// error of g is a sum of n random-walk errors of r: 3.6e-15 n^1.5 / sqrt(3),
// 2.4e-11 at n = 512, with a worst case of n^2 2^-48 / 2 = 4.7e-10);
// v = v_hi + v_lo is the float-float inverse PSD.  <d|h> sums float32 terms
// whose rounding errors are independent from bin to bin; the finalize bounds
// them by sum 3 and sends points over the tolerance to k_sg_refine.
constexpr int kSgSegment = kChunkMixed;

__device__ __forceinline__ void ff_mul_to(float& h, float& l, float bh, float bl) {
  const float p = __fmul_rn(h, bh);
  float e = __fmaf_rn(h, bh, -p);
  e = __fmaf_rn(h, bl, e);
  e = __fmaf_rn(l, bh, e);
  h = __fadd_rn(p, e);
  l = __fsub_rn(e, __fsub_rn(h, p));
}

// 64 points per CTA: twice the CTAs of the other mixed kernels, so that a
// batch of ten thousand points fills every SM with several CTAs
constexpr int kSgPointsPerCta = 64;

template <int D>
__global__ void __launch_bounds__(kSgPointsPerCta) k_mixed_sg(LaunchArgs a) {
  constexpr int CH = kChunkMixed;
  __shared__ __align__(16) float2 s_w[D][CH];
  __shared__ __align__(16) float s_vh[D][CH];
  __shared__ __align__(16) float s_vl[D][CH];
  __shared__ uint64_t bar;
  const int64_t k0 = a.k_base + (int64_t)blockIdx.y * CH;
  const int64_t slot = (int64_t)blockIdx.x * kSgPointsPerCta + threadIdx.x;
  const bool have = slot < a.B;
  const int64_t i = have && a.order ? (int64_t)a.order[slot] : slot;  // points ordered by centre frequency
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    mbar_fence_init();
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    mbar_expect_tx(&bar, D * CH * 16);
#pragma unroll
    for (int d = 0; d < D; ++d) {
      bulk_g2s(s_w[d], a.w[d] + k0, CH * 8, &bar);
      bulk_g2s(s_vh[d], a.v[d] + k0, CH * 4, &bar);
      bulk_g2s(s_vl[d], a.v_lo[d] + k0, CH * 4, &bar);
    }
  }
  const bool arrived = mbar_wait_bounded(&bar, 0, a.status, kWaitLimit);
  double t[D][4];
#pragma unroll
  for (int d = 0; d < D; ++d)
#pragma unroll
    for (int q = 0; q < 4; ++q) t[d][q] = 0.0;
  if (have && arrived && a.rec[i].valid) {
    const PointRec& r = a.rec[i];
    float ad[D], cd[D], a2h[D], a2l[D], c2h[D], c2l[D];
    uint32_t xl[D], xh[D];
#pragma unroll
    for (int d = 0; d < D; ++d) {
      const double A = r.fp[d] * r.amp, C = r.fx[d] * r.amp2, M = hypot(A, C);
      const double an = M > 0 ? A / M : 0.0, cn = M > 0 ? C / M : 0.0;
      ad[d] = (float)an;
      cd[d] = (float)cn;
      const ff q = ff_from_double(an * an), u = ff_from_double(cn * cn);
      a2h[d] = q.hi;
      a2l[d] = q.lo;
      c2h[d] = u.hi;
      c2l[d] = u.lo;
      xl[d] = r.xfix[d][0];
      xh[d] = r.xfix[d][1];
    }
    const double f0 = r.sg_f0, A = r.sg_a, df = a.step;
    const ff cc = ff_from_double(exp(-2.0 * A * df * df));
    // bins [0, ja) lie below the peak (walked downwards), [ja, CH) above it
    const double jp = floor((f0 - a.freq[k0]) / df);
    const int ja = (int)fmin(fmax(jp + 1.0, 0.0), (double)CH);
    for (int run = 0; run < 2; ++run) {
      const int dir = run == 0 ? 1 : -1;
      int j = run == 0 ? ja : ja - 1;
      int left = run == 0 ? CH - ja : ja;
      while (left > 0) {
        const int n = min(left, kSgSegment);
        // float64 start of the recurrence at bin j
        const double f = a.freq[k0 + j], x = f - f0, y = f + f0, st = dir * df;
        ff g1 = ff_from_double(exp(-A * x * x)), r1 = ff_from_double(exp(-A * (2.0 * x * st + df * df)));
        ff g2 = ff_from_double(exp(-A * y * y)), r2 = ff_from_double(exp(-A * (2.0 * y * st + df * df)));
        if (g1.hi == 0.f) r1.hi = r1.lo = 0.f;  // underflowed: stays zero (never inf * 0)
        if (g2.hi == 0.f) r2.hi = r2.lo = 0.f;
        float sr[D], cr[D], si[D], ci[D], hh[D], hl[D], e2[D];
#pragma unroll
        for (int d = 0; d < D; ++d) sr[d] = cr[d] = si[d] = ci[d] = hh[d] = hl[d] = e2[d] = 0.f;
        for (int q = 0; q < n; ++q, j += dir) {
          float hph = g1.hi, hpl = g1.lo, hxh = g1.hi, hxl = g1.lo;
          ff_add(hph, hpl, g2.hi, g2.lo);
          ff_add(hxh, hxl, -g2.hi, -g2.lo);
          // squares as unnormalised float-float pairs
          const float p2 = __fmul_rn(hph, hph), p2e = __fmaf_rn(2.f * hph, hpl, __fmaf_rn(hph, hph, -p2));
          const float x2 = __fmul_rn(hxh, hxh), x2e = __fmaf_rn(2.f * hxh, hxl, __fmaf_rn(hxh, hxh, -x2));
          const uint32_t k = (uint32_t)(k0 + j);
#pragma unroll
          for (int d = 0; d < D; ++d) {
            // The phase is linear in k: the accurate sincospi of the 0.32
            // fixed-point fraction rounded to float32, corrected to first
            // order by the exact integer residual of that rounding, so that
            // no approximation error repeats coherently and the phase error
            // is below 1e-14 rad.
            const int top = (int)(k * xh[d] + __umulhi(k, xl[d]));
            const float fc = __int2float_rn(top);
            const float eps = __int2float_rn((int)((long long)top - __float2ll_rz(fc))) * 1.4629180792671596e-09f;
            float sn, cs;
            sincospif(fc * 4.656612873077393e-10f, &sn, &cs);  // 2 pi top 2^-32 rad
            const float c1 = __fmaf_rn(-eps, sn, cs);
            sn = __fmaf_rn(eps, cs, sn);
            cs = c1;
            const float2 w = s_w[d][j];
            const float ere = w.x * cs - w.y * sn, eim = w.x * sn + w.y * cs;
            const float u = ad[d] * hph, z = cd[d] * hxh;
            kahan_add(sr[d], cr[d], u * ere - z * eim);
            kahan_add(si[d], ci[d], u * eim + z * ere);
            // (a^2 hp^2 + c^2 hx^2) v in float-float
            const float q1 = __fmul_rn(a2h[d], p2);
            float q1e = __fmaf_rn(a2h[d], p2, -q1);
            q1e = __fmaf_rn(a2h[d], p2e, __fmaf_rn(a2l[d], p2, q1e));
            const float q2 = __fmul_rn(c2h[d], x2);
            float q2e = __fmaf_rn(c2h[d], x2, -q2);
            q2e = __fmaf_rn(c2h[d], x2e, __fmaf_rn(c2l[d], x2, q2e));
            const float sh = __fadd_rn(q1, q2), sb = __fsub_rn(sh, q1);
            const float se = __fadd_rn(__fadd_rn(__fsub_rn(q1, __fsub_rn(sh, sb)), __fsub_rn(q2, sb)),
                                       __fadd_rn(q1e, q2e));
            ff_mac(hh[d], hl[d], sh, se, s_vh[d][j], s_vl[d][j]);
            // |term|^2 = (u^2 + z^2) |w|^2 (the rotation keeps the modulus)
            e2[d] = __fmaf_rn(__fmaf_rn(u, u, z * z), __fmaf_rn(w.x, w.x, w.y * w.y), e2[d]);
          }
          ff_mul_to(g1.hi, g1.lo, r1.hi, r1.lo);
          ff_mul_to(r1.hi, r1.lo, cc.hi, cc.lo);
          ff_mul_to(g2.hi, g2.lo, r2.hi, r2.lo);
          ff_mul_to(r2.hi, r2.lo, cc.hi, cc.lo);
        }
#pragma unroll
        for (int d = 0; d < D; ++d) {
          t[d][0] += (double)sr[d] - (double)cr[d];
          t[d][1] += (double)si[d] - (double)ci[d];
          t[d][2] += (double)hh[d] + (double)hl[d];
          t[d][3] += (double)e2[d];
        }
        left -= n;
      }
    }
  }
  if (have) {
#pragma unroll
    for (int d = 0; d < D; ++d)
#pragma unroll
      for (int q = 0; q < 4; ++q) a.part[(((int64_t)blockIdx.y * D + d) * kPartStride + q) * a.B + i] = t[d][q];
  }
}

// Sine-Gaussian points whose mixed-precision error bound exceeds the
// tolerance: float64 totals over the in-band bins (the plain kernel's
// arithmetic), one CTA per point, fixed-order reduction, then the point's
// lnL replaces the mixed one.
constexpr int kSgRefineThreads = 256;
__device__ void finish_point(const LaunchArgs& a, const PointRec& r, int64_t i, double dr, double di, double hh);

template <int D>
__global__ void __launch_bounds__(kSgRefineThreads) k_sg_refine(LaunchArgs a) {
  __shared__ double s_red[kSgRefineThreads / 32][3 * D];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t n = a.k_hi - a.k_lo, per = (n + kSgRefineThreads - 1) / kSgRefineThreads;
  for (int64_t i = blockIdx.x; i < a.B; i += gridDim.x) {
    const PointRec& r = a.rec[i];
    if (!r.refine) continue;  // the same i for the whole block
    const double f0 = r.sg_f0, amp = r.a[0], dplus = r.a[1], dcross = r.a[2], tau2 = r.a[3];
    const double pi2 = 9.869604401089358;
    double acc[3 * D];
#pragma unroll
    for (int q = 0; q < 3 * D; ++q) acc[q] = 0.0;
    const int64_t kb = a.k_lo + threadIdx.x * per, ke = min(kb + per, a.k_hi);
    if (kb < ke) {
      double zc[D], zs[D], rc[D], rs[D];
#pragma unroll
      for (int d = 0; d < D; ++d) {
        const double w2 = 2.0 * kPi * r.dt[d];
        sincos(w2 * a.freq[kb], &zs[d], &zc[d]);
        sincos(w2 * a.step, &rs[d], &rc[d]);
      }
      for (int64_t k = kb; k < ke; ++k) {
        const double f = a.freq[k];
        const double fm = f - f0, fpl = f + f0;
        const double neg = exp(-(fm * fm) * pi2 * tau2);
        const double pos = exp(-(fpl * fpl) * pi2 * tau2);
        const double hp = amp * (neg + pos) / dplus;
        const double hx_im = -(amp * (neg - pos) / dcross);
#pragma unroll
        for (int d = 0; d < D; ++d) {
          const double is = a.inv_psd[d][k];
          if (is != 0.0) {
            const double sre = hp * r.fp[d], sim = hx_im * r.fx[d];
            const double hre = sre * zc[d] + sim * zs[d], him = sim * zc[d] - sre * zs[d];
            const double2 dd = reinterpret_cast<const double2*>(a.strain[d])[k];
            acc[3 * d] += (hre * dd.x + him * dd.y) * is;
            acc[3 * d + 1] += (hre * dd.y - him * dd.x) * is;
            acc[3 * d + 2] += (hre * hre + him * him) * is;
          }
          rotate(zc[d], zs[d], rc[d], rs[d]);
        }
      }
    }
#pragma unroll
    for (int q = 0; q < 3 * D; ++q)
      for (int off = 16; off > 0; off >>= 1) acc[q] += __shfl_xor_sync(0xffffffffu, acc[q], off);
    if (lane == 0)
#pragma unroll
      for (int q = 0; q < 3 * D; ++q) s_red[warp][q] = acc[q];
    __syncthreads();
    if (threadIdx.x == 0) {
      const double norm = 4.0 / a.duration;
      double dr = 0.0, di = 0.0, hh = 0.0;
      for (int d = 0; d < D; ++d) {
        double x = 0.0, y = 0.0, z = 0.0;
        for (int w = 0; w < kSgRefineThreads / 32; ++w) {
          x += s_red[w][3 * d];
          y += s_red[w][3 * d + 1];
          z += s_red[w][3 * d + 2];
        }
        dr += norm * x;
        di += norm * y;
        hh += norm * z;
      }
      finish_point(a, r, i, dr, di, hh);
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// finalize: fixed-order reduction over chunks, <d|h>, <h|h>, marginalisation
// ---------------------------------------------------------------------------
__device__ __forceinline__ double neg_huge() { return -1.7976931348623157e308; }  // nan_to_num(-inf)

// p[t] = sum over groups c = 0, 1, ... (in that order) of the partial sums
// of detector d; the loads of 8 (or 4) groups are issued before their adds.
template <int NQ>
__device__ __forceinline__ void sum_groups(const LaunchArgs& a, int64_t i, int d, int64_t G, double* p) {
  constexpr int U = NQ <= 3 ? 8 : 4;
  const int64_t gs = (int64_t)a.n_det * kPartStride * a.B;
  const double* q = a.part + ((int64_t)d * kPartStride) * a.B + i;
  int64_t c = 0;
  for (; c + U <= G; c += U) {
    double v[U][NQ];
#pragma unroll
    for (int u = 0; u < U; ++u)
#pragma unroll
      for (int t = 0; t < NQ; ++t) v[u][t] = q[(c + u) * gs + (int64_t)t * a.B];
#pragma unroll
    for (int u = 0; u < U; ++u)
#pragma unroll
      for (int t = 0; t < NQ; ++t) p[t] += v[u][t];
  }
  for (; c < G; ++c)
#pragma unroll
    for (int t = 0; t < NQ; ++t) p[t] += q[c * gs + (int64_t)t * a.B];
}

// Error bound of the mixed sine-Gaussian lnL (k_mixed_sg).  Each <d|h> term
// carries six rounding errors of at most 2^-24 relative (the two weight
// components, the Gaussian's high word, sincospi's result, the product and
// the FMA), independent from bin to bin: an rms of about 8.5e-8 per term, so
// the sum errs by less than kSgRandomErr (4 sigma) times the Euclidean norm of
// the terms.  The float32 antenna factors add a coherent kSgCoherentErr
// |<d|h>|; the float-float <h|h> errs by less than kSgHhErr relative (the
// recurrence's worst case over a 512-bin walk is 4.7e-10).
constexpr double kSgRandomErr = 3.5e-7;
constexpr double kSgCoherentErr = 1e-7;
constexpr double kSgHhErr = 5e-10;

__device__ void detector_totals(const LaunchArgs& a, int64_t i, int64_t G, const PointRec& r, double* dh_re,
                                double* dh_im, double* hh, double* err = nullptr) {
  const double norm = 4.0 / a.duration;
  double sdr = 0.0, sdi = 0.0, shh = 0.0;
  for (int d = 0; d < a.n_det; ++d) {
    double p[kPartStride] = {0, 0, 0, 0, 0, 0};
    if (a.precision == GWL_PRECISION_FP64) {
      if (a.model == GWL_MODEL_SINEGAUSSIAN) sum_groups<3>(a, i, d, G, p);
      else sum_groups<2>(a, i, d, G, p);
    } else if (a.model == GWL_MODEL_SINEGAUSSIAN) sum_groups<4>(a, i, d, G, p);
    else if (a.cplx) sum_groups<2>(a, i, d, G, p);
    else sum_groups<1>(a, i, d, G, p);
    double dr, di, h;
    if (a.precision == GWL_PRECISION_FP64 && a.model == GWL_MODEL_SINEGAUSSIAN) {
      dr = norm * p[0];
      di = norm * p[1];
      h = norm * p[2];
    } else if (a.precision == GWL_PRECISION_FP64) {
      // <h|h> = A0^2 |Q|^2 sum_band f^(-7/3) / S
      dr = norm * p[0];
      di = norm * p[1];
      const double ci = r.cos_i;
      const double qr = r.fp[d] * (1.0 + ci * ci) / 2.0, qi = -r.fx[d] * ci;
      const int64_t k1 = min(r.k_end, a.n_bins), k0 = min(r.k_start, k1);
      h = norm * r.amp * r.amp * (qr * qr + qi * qi) * (a.hh_prefix[d][k1] - a.hh_prefix[d][k0]);
    } else if (a.model == GWL_MODEL_SINEGAUSSIAN) {
      // conj(h) = M (a hp + i c hx) e^{+i theta}, M = |(Fp P, Fx X)| (see k_mixed_sg)
      const double M = hypot(r.fp[d] * r.amp, r.fx[d] * r.amp2), ws = a.w_scale[d], vs = a.v_scale[d];
      dr = norm * ws * M * p[0];
      di = norm * ws * M * p[1];
      h = norm * vs * M * M * p[2];
      if (err) *err += kSgRandomErr * norm * ws * M * sqrt(fmax(p[3], 0.0));
    } else {
      // conj(h_det) = A0 f^(-7/6) conj(Q) e^{+i Phi},  Q = Fp (1 + c^2)/2 - i Fx c
      const double ci = r.cos_i;
      const double qr = r.fp[d] * (1.0 + ci * ci) / 2.0, qi = -r.fx[d] * ci;
      const double s = norm * a.w_scale[d] * r.amp;
      if (a.cplx) {
        // (qr - i qi) * (p0 + i p1)
        dr = s * (qr * p[0] + qi * p[1]);
        di = s * (qr * p[1] - qi * p[0]);
      } else {
        // p0 = Re sum w e^{i (phase + alpha_d)} (see PointRec::qfix)
        dr = s * r.qabs[d] * p[0];
        di = 0.0;
      }
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

// Components of a partial-sum record: <d|h> re/im and <h|h> (float64 kernels),
// the six sums of the sine-Gaussian mixed kernel, re/im for TaylorF2 mixed.
__device__ __host__ __forceinline__ int part_components(const LaunchArgs& a) {
  if (a.precision == GWL_PRECISION_FP64) return a.model == GWL_MODEL_SINEGAUSSIAN ? 3 : 2;
  return a.model == GWL_MODEL_SINEGAUSSIAN ? 4 : (a.cplx ? 2 : 1);
}

// One (point, detector, component) chain: the partial sums of all groups
// added in group order (loads of 8 groups in flight) into group 0's slot.
__device__ __forceinline__ void reduce_chain(const LaunchArgs& a, int64_t i, int d, int t) {
  const int64_t G = a.n_groups;
  const int64_t gs = (int64_t)a.n_det * kPartStride * a.B;
  double* q = a.part + ((int64_t)d * kPartStride + t) * a.B + i;
  double p = 0.0;
  int64_t c = 0;
  for (; c + 8 <= G; c += 8) {
    double v[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) v[u] = q[(c + u) * gs];
#pragma unroll
    for (int u = 0; u < 8; ++u) p += v[u];
  }
  for (; c < G; ++c) p += q[c * gs];
  q[0] = p;
}

__global__ void k_reduce_parts(LaunchArgs a) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int nq = part_components(a);
  if (idx >= a.B * a.n_det * nq) return;
  const int64_t i = idx % a.B, r = idx / a.B;
  reduce_chain(a, i, (int)(r / nq), (int)(r % nq));
}

// lnL of point i from its totals <d|h> = dr + i di and <h|h> (base.py:448-477
// without time marginalisation), with the optional outputs of the totals.
__device__ void finish_point(const LaunchArgs& a, const PointRec& r, int64_t i, double dr, double di, double hh) {
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

// G: the groups still to be summed (1 after k_reduce_parts)
__device__ __noinline__ void finalize_point(const LaunchArgs& a, int64_t i, int64_t G) {
  const PointRec& r = a.rec[i];
  double dr, di, hh, err = 0.0;
  const bool sg_bound = a.model == GWL_MODEL_SINEGAUSSIAN && a.precision == GWL_PRECISION_MIXED && a.rf_tol > 0 &&
                        a.rf_count && r.valid;
  detector_totals(a, i, G, r, &dr, &di, &hh, sg_bound ? &err : nullptr);
  finish_point(a, r, i, dr, di, hh);
  if (sg_bound) {
    // the bound holds for Re <d|h> - <h|h> / 2 and, as ln I0 has slope at
    // most one, for the phase-marginalised ln I0(|<d|h>|) - <h|h> / 2; with
    // the distance table the slopes are at most r and r^2 / 2 (r = dist_slope)
    const double slope = a.dist_slope > 1.0 ? a.dist_slope : 1.0;
    err = slope * (err + kSgCoherentErr * (fabs(dr) + fabs(di))) + slope * slope * kSgHhErr * hh;
    if (!(err <= a.rf_tol)) {
      a.rec[i].refine = 1;
      atomicAdd(a.rf_count, 1);
    }
  }
}

// ---------------------------------------------------------------------------
// relative binning (bilby/gw/likelihood/relative.py:365-402)
// ---------------------------------------------------------------------------
// One warp per point.  Lane l evaluates the model at edge e = 31 q + l (q-th
// pass), projects it on each detector, multiplies by 1 / h0_d(f_e) and takes
// the ratio at edge e + 1 from lane l + 1; lanes 0..30 then add bin e's terms
//   <d|h> += a0 conj(r0) + a1 conj(r1),  <h|h> += b0 |r0|^2 + 2 b1 Re(r0 conj(r1))
// with r0 = (r_{e+1} + r_e) / 2 and r1 = (r_{e+1} - r_e) / (f_{e+1} - f_e).
// float64 throughout.
constexpr int kRelbinWarps = 4;

template <int D>
__global__ void __launch_bounds__(32 * kRelbinWarps) k_relbin(LaunchArgs a) {
  const int lane = threadIdx.x & 31;
  const int64_t i = (int64_t)blockIdx.x * kRelbinWarps + (threadIdx.x >> 5);
  if (i >= a.B) return;  // uniform over the warp
  const PointRec& r = a.rec[i];
  const int nE = a.rb_edges, nB = nE - 1;
  double dre = 0.0, dim = 0.0, hh = 0.0;
  if (r.valid) {
    double fp[D], fx[D], w2[D];
#pragma unroll
    for (int d = 0; d < D; ++d) {
      fp[d] = r.fp[d];
      fx[d] = r.fx[d];
      w2[d] = 2.0 * kPi * r.dt[d];
    }
    const bool tf2 = a.model == GWL_MODEL_TAYLORF2;
    const double u = tf2 ? cbrt(kPi * r.m_sec) : 0.0, lnu = tf2 ? log(u) : 0.0;
    const double pu5 = tf2 ? 3.0 / (128.0 * r.eta) / (u * u * u * u * u) : 0.0;
    const double ci = r.cos_i, pfac = (1.0 + ci * ci) / 2.0;
    for (int base = 0; base < nB; base += 31) {
      const int e = base + lane;
      double rr[D], ri[D];
#pragma unroll
      for (int d = 0; d < D; ++d) rr[d] = ri[d] = 0.0;
      if (e < nE) {
        const double f = a.rb_freq[e];
        double hpr = 0.0, hpi = 0.0, hxr = 0.0, hxi = 0.0;
        if (tf2) {
          if (f >= a.fmin && f < r.f_isco) {
            const double4 t = a.ftab[a.rb_index[e]];
            const double v = u * t.x, lnv = lnu + t.y;
            double sm = r.a[7];
#pragma unroll
            for (int q = 6; q >= 0; --q) sm = sm * v + r.a[q];
            const double v5 = v * v * v * v * v;
            sm = sm + lnv * (r.l[5] + r.l[6] * v) * v5;
            const double psi = (-2.0 * r.phase - kPi / 4) + pu5 * sm * t.z;
            const double amp = r.amp * t.w;
            double sp, cp;
            sincos(psi, &sp, &cp);
            const double ere = amp * cp, eim = -amp * sp;
            hpr = pfac * ere;
            hpi = pfac * eim;
            hxr = ci * eim;
            hxi = -ci * ere;
          }
        } else {
          // source.py:1199-1207
          const double pi2 = 9.869604401089358;
          const double fm = f - r.sg_f0, fpl = f + r.sg_f0;
          const double neg = exp(-(fm * fm) * pi2 * r.a[3]);
          const double pos = exp(-(fpl * fpl) * pi2 * r.a[3]);
          hpr = r.a[0] * (neg + pos) / r.a[1];
          hxi = -(r.a[0] * (neg - pos) / r.a[2]);
        }
#pragma unroll
        for (int d = 0; d < D; ++d) {
          // interferometer.py:341-362 at explicit frequencies (no mask)
          const double sre = hpr * fp[d] + hxr * fx[d];
          const double sim = hpi * fp[d] + hxi * fx[d];
          double sn, cs;
          sincos(w2[d] * f, &sn, &cs);
          const double hre = sre * cs + sim * sn, him = sim * cs - sre * sn;
          const double2 g = a.rb_h0inv[d][e];
          rr[d] = hre * g.x - him * g.y;
          ri[d] = hre * g.y + him * g.x;
        }
      }
      const bool bin = lane < 31 && e < nB;
      const double width = bin ? a.rb_freq[e + 1] - a.rb_freq[e] : 1.0;
#pragma unroll
      for (int d = 0; d < D; ++d) {
        const double nr = __shfl_down_sync(0xffffffffu, rr[d], 1);
        const double ni = __shfl_down_sync(0xffffffffu, ri[d], 1);
        if (bin) {
          const double r0r = (nr + rr[d]) / 2, r0i = (ni + ri[d]) / 2;
          const double r1r = (nr - rr[d]) / width, r1i = (ni - ri[d]) / width;
          const double* sd = a.rb_sum[d] + (size_t)e * 6;
          const double a0r = sd[0], a0i = sd[1], a1r = sd[2], a1i = sd[3], b0 = sd[4], b1 = sd[5];
          dre += a0r * r0r + a0i * r0i + a1r * r1r + a1i * r1i;
          dim += a0i * r0r - a0r * r0i + a1i * r1r - a1r * r1i;
          hh += b0 * (r0r * r0r + r0i * r0i) + 2.0 * b1 * (r0r * r1r + r0i * r1i);
        }
      }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      dre += __shfl_xor_sync(0xffffffffu, dre, off);
      dim += __shfl_xor_sync(0xffffffffu, dim, off);
      hh += __shfl_xor_sync(0xffffffffu, hh, off);
    }
  }
  if (lane == 0) finish_point(a, r, i, dre, dim, hh);
}

// The float64 TaylorF2 or sine-Gaussian polarisations at one frequency, the
// TaylorF2 powers of f from a table entry t.
struct PointModel {
  bool tf2;
  double u, lnu, pu5, ci, pfac;
};

__device__ __forceinline__ PointModel point_model(const LaunchArgs& a, const PointRec& r) {
  PointModel m;
  m.tf2 = a.model == GWL_MODEL_TAYLORF2;
  m.u = m.tf2 ? cbrt(kPi * r.m_sec) : 0.0;
  m.lnu = m.tf2 ? log(m.u) : 0.0;
  m.pu5 = m.tf2 ? 3.0 / (128.0 * r.eta) / (m.u * m.u * m.u * m.u * m.u) : 0.0;
  m.ci = r.cos_i;
  m.pfac = (1.0 + m.ci * m.ci) / 2.0;
  return m;
}

__device__ __forceinline__ void model_at(const LaunchArgs& a, const PointRec& r, const PointModel& m, double f,
                                         const double4& t, double& hpr, double& hpi, double& hxr, double& hxi) {
  hpr = hpi = hxr = hxi = 0.0;
  if (m.tf2) {
    if (f >= a.fmin && f < r.f_isco) {
      const double v = m.u * t.x, lnv = m.lnu + t.y;
      double sm = r.a[7];
#pragma unroll
      for (int q = 6; q >= 0; --q) sm = sm * v + r.a[q];
      const double v5 = v * v * v * v * v;
      sm = sm + lnv * (r.l[5] + r.l[6] * v) * v5;
      const double psi = (-2.0 * r.phase - kPi / 4) + m.pu5 * sm * t.z;
      const double amp = r.amp * t.w;
      double sp, cp;
      sincos(psi, &sp, &cp);
      const double ere = amp * cp, eim = -amp * sp;
      hpr = m.pfac * ere;
      hpi = m.pfac * eim;
      hxr = m.ci * eim;
      hxi = -m.ci * ere;
    }
  } else {
    const double pi2 = 9.869604401089358;
    const double fm = f - r.sg_f0, fpl = f + r.sg_f0;
    const double neg = exp(-(fm * fm) * pi2 * r.a[3]);
    const double pos = exp(-(fpl * fpl) * pi2 * r.a[3]);
    hpr = r.a[0] * (neg + pos) / r.a[1];
    hxi = -(r.a[0] * (neg - pos) / r.a[2]);
  }
}

// ---------------------------------------------------------------------------
// reduced-order quadrature (bilby/gw/likelihood/roq.py:467-602, one basis,
// no time marginalisation): one warp per point.  Lanes stride over the
// linear nodes, accumulating for each detector the five sums
//   D_m = sum_j conj(h_d(F_j)) W_d[c + m - 2][j],  m = 0..4,
// at the time samples around the detector's arrival time (c the closest
// sample below it), then over the quadratic nodes for
//   <h|h> += sum_j |h_d(G_j)|^2 w_d[j].
// Lane 0 interpolates the five D_m to the arrival time (LIGO-T2100224).  The
// detector time shift lives in the weights, so h carries no e^{-2 pi i f dt}.
// float64 throughout.
// ---------------------------------------------------------------------------
template <int D>
__global__ void __launch_bounds__(32 * kRelbinWarps) k_roq(LaunchArgs a) {
  const int lane = threadIdx.x & 31;
  const int64_t i = (int64_t)blockIdx.x * kRelbinWarps + (threadIdx.x >> 5);
  if (i >= a.B) return;  // uniform over the warp
  const PointRec& r = a.rec[i];
  double dr = 0.0, di = 0.0, hh = 0.0;
  if (r.valid) {
    double fp[D], fx[D], ar[D][5], ai[D][5], tifo[D];
    int64_t row[D][5];
    bool inb[D];
    const double t0 = (double)a.roq_time_start * a.roq_dt;
    const double step = (double)(a.roq_time_start + 1) * a.roq_dt - t0;
#pragma unroll
    for (int d = 0; d < D; ++d) {
      fp[d] = r.fp[d];
      fx[d] = r.fx[d];
      // the detector's arrival time after the segment start: with time
      // marginalisation dt holds the delay at the antenna time alone and the
      // jitter enters only the time series (roq.py:529-541: geocent_time as
      // given, minus the start, plus that delay)
      tifo[d] = a.roq_tm ? (par(a, GWL_P_GEOCENT_TIME, i) - a.det[d].start_time) + r.dt[d] : r.dt[d];
      // roq.py:552-575: the five samples around the arrival time
      const int64_t c = (int64_t)floor((tifo[d] - t0) / step);
      inb[d] = c - 2 >= 0 && c + 2 < a.roq_n_time;
#pragma unroll
      for (int m = 0; m < 5; ++m) {
        const int64_t k = c + m - 2;
        row[d][m] = k < 0 ? 0 : (k > a.roq_n_time - 1 ? a.roq_n_time - 1 : k);
        ar[d][m] = ai[d][m] = 0.0;
      }
    }
    const PointModel pm = point_model(a, r);
    for (int j = lane; j < a.roq_nl; j += 32) {
      double hpr, hpi, hxr, hxi;
      model_at(a, r, pm, a.roq_fl[j], a.roq_pl[j], hpr, hpi, hxr, hxi);
#pragma unroll
      for (int d = 0; d < D; ++d) {
        const double hr = hpr * fp[d] + hxr * fx[d], hi = hpi * fp[d] + hxi * fx[d];
#pragma unroll
        for (int m = 0; m < 5; ++m) {
          const double2 w = a.roq_wl[d][row[d][m] * a.roq_nl + j];
          // conj(h) w
          ar[d][m] += hr * w.x + hi * w.y;
          ai[d][m] += hr * w.y - hi * w.x;
        }
      }
    }
    for (int j = lane; j < a.roq_nq; j += 32) {
      double hpr, hpi, hxr, hxi;
      model_at(a, r, pm, a.roq_fq[j], a.roq_pq[j], hpr, hpi, hxr, hxi);
#pragma unroll
      for (int d = 0; d < D; ++d) {
        const double hr = hpr * fp[d] + hxr * fx[d], hi = hpi * fp[d] + hxi * fx[d];
        hh += (hr * hr + hi * hi) * a.roq_wq[d][j];
      }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      hh += __shfl_xor_sync(0xffffffffu, hh, off);
#pragma unroll
      for (int d = 0; d < D; ++d)
#pragma unroll
        for (int m = 0; m < 5; ++m) {
          ar[d][m] += __shfl_xor_sync(0xffffffffu, ar[d][m], off);
          ai[d][m] += __shfl_xor_sync(0xffffffffu, ai[d][m], off);
        }
    }
    // roq.py:577-602 on the (clipped) sample times; out of range: + log(0)
#pragma unroll
    for (int d = 0; d < D; ++d) {
      const double ts0 = (double)(a.roq_time_start + row[d][0]) * a.roq_dt;
      const double ts1 = (double)(a.roq_time_start + row[d][1]) * a.roq_dt;
      const double ts3 = (double)(a.roq_time_start + row[d][3]) * a.roq_dt;
      const double aa = (ts3 - tifo[d]) / fmax(ts1 - ts0, 1e-12);
      const double bb = 1.0 - aa;
      const double cc = (aa * aa * aa - aa) / 6.0, dd = (bb * bb * bb - bb) / 6.0;
      const double r1r = (-ar[d][0] + 8.0 * ar[d][1] - 14.0 * ar[d][2] + 8.0 * ar[d][3] - ar[d][4]) / 4.0;
      const double r1i = (-ai[d][0] + 8.0 * ai[d][1] - 14.0 * ai[d][2] + 8.0 * ai[d][3] - ai[d][4]) / 4.0;
      const double r2r = ar[d][2] - 2.0 * ar[d][3] + ar[d][4], r2i = ai[d][2] - 2.0 * ai[d][3] + ai[d][4];
      dr += aa * ar[d][2] + bb * ar[d][3] + cc * r1r + dd * r2r + (inb[d] ? 0.0 : -INFINITY);
      di += aa * ai[d][2] + bb * ai[d][3] + cc * r1i + dd * r2i;
    }
  }
  if (lane == 0) finish_point(a, r, i, dr, di, hh);
}

// ---------------------------------------------------------------------------
// multi-banding (bilby/gw/likelihood/multiband.py:741-819, linear
// interpolation of <h|h>): one warp per point, lanes striding over the banded
// frequencies; <d|h> = conj(sum_k s_k L_k), <h|h> = sum_k |s_k|^2 Q_k with the
// detector response s_k at banded frequency k.  float64 throughout.
// ---------------------------------------------------------------------------
template <int D>
__global__ void __launch_bounds__(32 * kRelbinWarps) k_multiband(LaunchArgs a) {
  const int lane = threadIdx.x & 31;
  const int64_t i = (int64_t)blockIdx.x * kRelbinWarps + (threadIdx.x >> 5);
  if (i >= a.B) return;  // uniform over the warp
  const PointRec& r = a.rec[i];
  if (a.mb_refine_only && !r.refine) return;  // uniform over the warp
  double sr = 0.0, si = 0.0, hh = 0.0;
  if (r.valid) {
    double fp[D], fx[D], w2[D];
#pragma unroll
    for (int d = 0; d < D; ++d) {
      fp[d] = r.fp[d];
      fx[d] = r.fx[d];
      w2[d] = 2.0 * kPi * r.dt[d];
    }
    const PointModel m = point_model(a, r);
    // inside a band the banded frequencies are uniform (spacing df_b): this
    // lane's e^{i w f} advances by e^{i w 32 df_b} from point to point
    for (int b = 0; b < a.mb_bands; ++b) {
      const int64_t k0 = a.mb_band_start[b] + lane, k1 = a.mb_band_start[b + 1];
      if (k0 >= k1) continue;
      double zc[D], zs[D], rc[D], rs[D];
#pragma unroll
      for (int d = 0; d < D; ++d) {
        sincos(w2[d] * a.mb_freq[k0], &zs[d], &zc[d]);
        sincos(w2[d] * (32.0 * a.mb_band_df[b]), &rs[d], &rc[d]);
      }
      for (int64_t k = k0; k < k1; k += 32) {
        const double f = a.mb_freq[k];
        double hpr, hpi, hxr, hxi;
        model_at(a, r, m, f, a.mb_pow[k], hpr, hpi, hxr, hxi);
        if (hpr != 0.0 || hpi != 0.0 || hxr != 0.0 || hxi != 0.0) {
#pragma unroll
          for (int d = 0; d < D; ++d) {
            const double sre = hpr * fp[d] + hxr * fx[d];
            const double sim = hpi * fp[d] + hxi * fx[d];
            const double sn = zs[d], cs = zc[d];
            const double hre = sre * cs + sim * sn, him = sim * cs - sre * sn;
            const double2 L = a.mb_lin[d][k];
            sr += hre * L.x - him * L.y;
            si += hre * L.y + him * L.x;
            hh += (hre * hre + him * him) * a.mb_quad[d][k];
          }
        }
#pragma unroll
        for (int d = 0; d < D; ++d) rotate(zc[d], zs[d], rc[d], rs[d]);
      }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      sr += __shfl_xor_sync(0xffffffffu, sr, off);
      si += __shfl_xor_sync(0xffffffffu, si, off);
      hh += __shfl_xor_sync(0xffffffffu, hh, off);
    }
  }
  if (lane == 0 && r.valid) hh += mb_fft_hh_total(a, i);
  // <d|h> = conj(sum s L)
  if (lane == 0) finish_point(a, r, i, sr, -si, hh);
}

// Multi-banding in mixed precision: one warp per point, lanes over the banded
// frequencies of each band.  The phase of every banded frequency comes from
// the float-float basis at that frequency (mb_basis) reduced to 0.64 fixed
// point; detector d's time shift f dt_d is exact in 0.64 fixed point per band
// (frac(f_b0 dt_d) + i frac(df_b dt_d), f = f_b0 + i df_b); cos / sin by the
// hardware approximation; the linear coefficients times f^(-7/6) in float32;
// 8-term float32 partials folded into float-float, then float64 over the
// warp.  <h|h> needs no per-frequency work: A^2 |Q_d|^2 times the prefix sum
// of f^(-7/3) quad over the point's band.
constexpr double kMbRandomErr = 1e-6;

template <int D>
__global__ void __launch_bounds__(32 * kRelbinWarps) k_multiband_mixed(LaunchArgs a) {
  const int lane = threadIdx.x & 31;
  const int64_t i = (int64_t)blockIdx.x * kRelbinWarps + (threadIdx.x >> 5);
  if (i >= a.B) return;  // uniform over the warp
  const PointRec& r = a.rec[i];
  double sr = 0.0, si = 0.0, hh = 0.0;
  if (r.valid) {
    // the point's band among the banded frequencies: fmin <= f < f_isco
    int64_t kb0 = 0, kb1 = a.mb_points;
    {
      int64_t lo = 0, hi = a.mb_points;
      while (lo < hi) {
        const int64_t mid = (lo + hi) / 2;
        if (a.mb_freq[mid] >= a.fmin) hi = mid; else lo = mid + 1;
      }
      kb0 = lo;
      lo = kb0;
      hi = a.mb_points;
      while (lo < hi) {
        const int64_t mid = (lo + hi) / 2;
        if (a.mb_freq[mid] >= r.f_isco) hi = mid; else lo = mid + 1;
      }
      kb1 = lo;
    }
    float ch[kNumBasis + 1], cl[kNumBasis + 1];
#pragma unroll
    for (int b = 0; b <= kNumBasis; ++b) {
      ch[b] = r.c_hi[b];
      cl[b] = r.c_lo[b];
    }
    float ahi[D], alo[D], bhi[D], blo[D], pre[D], pim[D];
#pragma unroll
    for (int d = 0; d < D; ++d) ahi[d] = alo[d] = bhi[d] = blo[d] = pre[d] = pim[d] = 0.f;
    int n_acc = 0;
    for (int b = 0; b < a.mb_bands; ++b) {
      const int64_t bs = a.mb_band_start[b];
      const int64_t k_lo = max(bs, kb0), k_hi = min(a.mb_band_start[b + 1], kb1);
      if (k_lo >= k_hi) continue;  // uniform over the warp
      // detector d's shift in this band, 0.64 fixed point: lane d computes it
      uint64_t Yl = 0, Xl = 0;
      if (lane < D) {
        const double dt = r.dt[lane];
        const double y = a.mb_freq[bs] * dt, x = a.mb_band_df[b] * dt;
        double fy = ldexp(y - floor(y), 64), fx = ldexp(x - floor(x), 64);
        if (!(fy < 18446744073709551616.0)) fy = 0.0;
        if (!(fx < 18446744073709551616.0)) fx = 0.0;
        Yl = (uint64_t)fy;
        Xl = (uint64_t)fx;
      }
      uint64_t Y[D], X[D];
#pragma unroll
      for (int d = 0; d < D; ++d) {
        Y[d] = __shfl_sync(0xffffffffu, Yl, d);
        X[d] = __shfl_sync(0xffffffffu, Xl, d);
      }
      for (int64_t k = k_lo + lane; k < k_hi; k += 32) {
        const float4* bp = reinterpret_cast<const float4*>(a.mb_basis + k * kNumBasis);
        float s_hi = ch[kNumBasis], s_lo = cl[kNumBasis];
#pragma unroll
        for (int q = 0; q < kNumBasis / 2; ++q) {
          const float4 v = __ldg(bp + q);
          ff_mac(s_hi, s_lo, ch[2 * q], cl[2 * q], v.x, v.y);
          ff_mac(s_hi, s_lo, ch[2 * q + 1], cl[2 * q + 1], v.z, v.w);
        }
        const uint64_t base = to_fixed(s_hi, s_lo);
        const uint64_t idx = (uint64_t)(k - bs);
#pragma unroll
        for (int d = 0; d < D; ++d) {
          const uint64_t full = base + Y[d] + idx * X[d];
          const uint32_t top = (uint32_t)((full + 0x80000000ull) >> 32);
          // sincospi of the exact fraction (cycles in [-1/2, 1/2)): rounding
          // errors independent from term to term, bounded in the epilogue
          const float ph = __fmul_rn(__int2float_rn((int)top), 4.656612873077393e-10f);  // 2 * 2^-32
          float sn, cs;
          sincospif(ph, &sn, &cs);
          const float2 L = __ldg(a.mb_lw[d] + k);
          // h_d L with h_d proportional to exp(-i phase)
          pre[d] = __fmaf_rn(cs, L.x, __fmaf_rn(sn, L.y, pre[d]));
          pim[d] = __fmaf_rn(cs, L.y, __fmaf_rn(-sn, L.x, pim[d]));
        }
        if (++n_acc == 8) {
#pragma unroll
          for (int d = 0; d < D; ++d) {
            two_sum_acc(ahi[d], alo[d], pre[d]);
            two_sum_acc(bhi[d], blo[d], pim[d]);
            pre[d] = pim[d] = 0.f;
          }
          n_acc = 0;
        }
      }
    }
    double P_re[D], P_im[D];
#pragma unroll
    for (int d = 0; d < D; ++d) {
      two_sum_acc(ahi[d], alo[d], pre[d]);
      two_sum_acc(bhi[d], blo[d], pim[d]);
      P_re[d] = (double)ahi[d] + (double)alo[d];
      P_im[d] = (double)bhi[d] + (double)blo[d];
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) {
        P_re[d] += __shfl_xor_sync(0xffffffffu, P_re[d], off);
        P_im[d] += __shfl_xor_sync(0xffffffffu, P_im[d], off);
      }
    }
    if (lane == 0) {
      // sum_d A Q_d P_d scale_d, Q_d = Fp (1 + c^2) / 2 - i Fx c
      const double ci = r.cos_i, pfac = (1.0 + ci * ci) / 2.0;
      double err = 0.0;
      for (int d = 0; d < D; ++d) {
        const double qr = r.fp[d] * pfac, qi = -r.fx[d] * ci;
        const double pr = P_re[d] * a.mb_lw_scale[d], pm = P_im[d] * a.mb_lw_scale[d];
        sr += r.amp * (qr * pr - qi * pm);
        si += r.amp * (qr * pm + qi * pr);
        hh += r.amp * r.amp * (qr * qr + qi * qi) * (a.mb_qprefix[d][kb1] - a.mb_qprefix[d][kb0]);
        // float32 terms with independent relative errors below about 2.5e-7
        // (the phase fraction, sincospi, the weight, two FMAs): kMbRandomErr
        // (a 4-sigma margin) times their Euclidean norm
        err += kMbRandomErr * r.amp * hypot(qr, qi) * a.mb_lw_scale[d] *
               sqrt(fmax(a.mb_l2prefix[d][kb1] - a.mb_l2prefix[d][kb0], 0.0));
      }
      // (times the distance slope bound: the lnL's change per unit <d|h>)
      if (a.dist_slope > 1.0) err *= a.dist_slope;
      if (a.rf_tol > 0 && a.rf_count && !(err <= a.rf_tol)) {
        a.rec[i].refine = 1;
        atomicAdd(a.rf_count, 1);
      }
    }
  }
  if (lane == 0 && r.valid) hh += mb_fft_hh_total(a, i);
  // <d|h> = conj(sum h L)
  if (lane == 0) finish_point(a, r, i, sr, -si, hh);
}

__global__ void k_finalize(LaunchArgs a) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.B) return;
  finalize_point(a, i, 1);
}


// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
// The per-point float64 steps run one warp per CTA so that a batch of a few
// thousand points spreads over all SMs (their float64 pipes bound them).
constexpr int kPointThreads = 32;

cudaError_t launch_prologue(const LaunchArgs& a, cudaStream_t s) {
  const int threads = kPointThreads;
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
constexpr auto k_mixed_tf2_c = k_mixed_tf2<D, true>;
template <int D>
constexpr auto k_mixed_tf2_r = k_mixed_tf2<D, false>;
template <int D>
constexpr auto k_mixed_tf2_acc_c = k_mixed_tf2_acc<D, true>;
template <int D>
constexpr auto k_mixed_tf2_acc_r = k_mixed_tf2_acc<D, false>;

// resident CTAs per SM of the accurate kernel, per detector count
static int acc_ctas_per_sm[kMaxDet + 1] = {};

template <int D>
static cudaError_t set_mixed_smem() {
  const int bytes = 2 * D * kChunkMixed * 8;
  cudaError_t e = cudaFuncSetAttribute(k_mixed_tf2<D, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e != cudaSuccess) return e;
  if ((e = cudaFuncSetAttribute(k_mixed_tf2<D, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes)) !=
      cudaSuccess)
    return e;
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_mixed_tf2_acc<D, false>, kAccThreads, 0) != cudaSuccess ||
      n < 1)
    n = 1;
  acc_ctas_per_sm[D] = n;
  return cudaSuccess;
}

static int sm_count_k() {
  static int n = 0;
  if (n == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    if (n <= 0) n = 152;
  }
  return n;
}

// shared-memory limits and occupancies of the mixed TaylorF2 kernels, once
// per process (a function-local static: initialised once even when several
// host threads make their first launches at the same time)
static cudaError_t configure_mixed() {
  static const cudaError_t status = [] {
    cudaError_t e;
    if ((e = set_mixed_smem<1>()) != cudaSuccess) return e;
    if ((e = set_mixed_smem<2>()) != cudaSuccess) return e;
    if ((e = set_mixed_smem<3>()) != cudaSuccess) return e;
    return set_mixed_smem<4>();
  }();
  return status;
}

cudaError_t launch_mixed(const LaunchArgs& a, cudaStream_t s) {
  if (a.model == GWL_MODEL_SINEGAUSSIAN) {
    dim3 grid((unsigned)((a.B + kSgPointsPerCta - 1) / kSgPointsPerCta), (unsigned)a.n_chunks);
    GWL_DISPATCH_D(k_mixed_sg, grid, kSgPointsPerCta, 0, s, a);
  } else {
    const cudaError_t ce = configure_mixed();
    if (ce != cudaSuccess) return ce;
    dim3 grid((unsigned)((a.B + kPointsPerCta - 1) / kPointsPerCta), (unsigned)a.n_groups);
    const int smem = 2 * a.n_det * kChunkMixed * 8;
    if (a.cplx) {
      GWL_DISPATCH_D(k_mixed_tf2_c, grid, kPointsPerCta, smem, s, a);
    } else {
      GWL_DISPATCH_D(k_mixed_tf2_r, grid, kPointsPerCta, smem, s, a);
    }
  }
  return cudaGetLastError();
}

cudaError_t launch_mixed_acc(const LaunchArgs& a, cudaStream_t s) {
  if (a.model != GWL_MODEL_TAYLORF2 || !(a.rf_tol > 0) || !a.rf_count || !a.order || a.B <= 0) return cudaSuccess;
  {
    const cudaError_t ce = configure_mixed();
    if (ce != cudaSuccess) return ce;
    // the marked points (first slots of the ordering), one warp per (point, group)
    const int64_t warps = a.B * a.n_groups;
    const unsigned g_acc = (unsigned)min((warps + kAccThreads / 32 - 1) / (kAccThreads / 32),
                                         (int64_t)sm_count_k() * acc_ctas_per_sm[min(a.n_det, kMaxDet)]);
    if (a.cplx) {
      GWL_DISPATCH_D(k_mixed_tf2_acc_c, g_acc, kAccThreads, 0, s, a);
    } else {
      GWL_DISPATCH_D(k_mixed_tf2_acc_r, g_acc, kAccThreads, 0, s, a);
    }
  }
  return cudaGetLastError();
}

// Group sums in parallel over (point, detector, component), then the
// per-point totals and marginalisation.
cudaError_t launch_finalize(const LaunchArgs& a, cudaStream_t s) {
  const int64_t chains = a.B * a.n_det * part_components(a);
  k_reduce_parts<<<(unsigned)((chains + 127) / 128), 128, 0, s>>>(a);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  const int threads = kPointThreads;
  k_finalize<<<(unsigned)((a.B + threads - 1) / threads), threads, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_sg_refine(const LaunchArgs& a, cudaStream_t s) {
  if (a.model != GWL_MODEL_SINEGAUSSIAN || !(a.rf_tol > 0) || !a.rf_count || a.B <= 0) return cudaSuccess;
  const unsigned grid = (unsigned)min(a.B, (int64_t)4 * sm_count_k());
  GWL_DISPATCH_D(k_sg_refine, grid, kSgRefineThreads, 0, s, a);
  return cudaGetLastError();
}

cudaError_t launch_roq(const LaunchArgs& a, cudaStream_t s) {
  const unsigned grid = (unsigned)((a.B + kRelbinWarps - 1) / kRelbinWarps);
  GWL_DISPATCH_D(k_roq, grid, 32 * kRelbinWarps, 0, s, a);
  return cudaGetLastError();
}

cudaError_t launch_multiband_mixed(const LaunchArgs& a, cudaStream_t s) {
  const unsigned grid = (unsigned)((a.B + kRelbinWarps - 1) / kRelbinWarps);
  GWL_DISPATCH_D(k_multiband_mixed, grid, 32 * kRelbinWarps, 0, s, a);
  return cudaGetLastError();
}

cudaError_t launch_multiband(const LaunchArgs& a, cudaStream_t s) {
  const unsigned grid = (unsigned)((a.B + kRelbinWarps - 1) / kRelbinWarps);
  GWL_DISPATCH_D(k_multiband, grid, 32 * kRelbinWarps, 0, s, a);
  return cudaGetLastError();
}

cudaError_t launch_relbin(const LaunchArgs& a, cudaStream_t s) {
  const unsigned grid = (unsigned)((a.B + kRelbinWarps - 1) / kRelbinWarps);
  GWL_DISPATCH_D(k_relbin, grid, 32 * kRelbinWarps, 0, s, a);
  return cudaGetLastError();
}

void order_layout(int64_t n_chunks, int* keys, int* shift) {
  int sh = 0;
  while ((n_chunks >> sh) + 1 > kOrderMaxKeys) ++sh;
  *shift = sh;
  *keys = (int)(n_chunks >> sh) + 1;
}

void ordering_by_peak(LaunchArgs& L) {
  int keys = 0, shift = 0;
  order_layout(L.n_chunks * L.chunk, &keys, &shift);
  L.order_shift = shift;
  L.order_half = 0;
  L.order_keys = keys;
  L.rf_count = L.order_hist ? L.order_hist + 2 * L.order_keys : nullptr;
}

void ordering_with_marks(LaunchArgs& L) {
  int keys = 0, shift = 0;
  order_layout(L.n_chunks, &keys, &shift);
  L.order_shift = shift;
  L.order_half = L.rf_tol > 0 ? keys : 0;
  L.order_keys = L.rf_tol > 0 ? 2 * keys : keys;
  L.rf_count = L.order_hist ? L.order_hist + 2 * L.order_keys : nullptr;
}

// Bases of the buckets counted by the prologue, then each point's slot.
cudaError_t launch_order(const LaunchArgs& a, cudaStream_t s) {
  k_order_scan<<<1, kOrderThreads, 0, s>>>(a);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  const int threads = 128;
  k_order_scatter<<<(unsigned)((a.B + threads - 1) / threads), threads, 0, s>>>(a);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// several analyses in one launch sequence
// ---------------------------------------------------------------------------
__device__ __forceinline__ int find_item(const int64_t* off, int n, int64_t p) {
  int lo = 0, hi = n - 1;  // largest item with off[item] <= p
  while (lo < hi) {
    const int mid = (lo + hi + 1) / 2;
    if (off[mid] <= p) lo = mid; else hi = mid - 1;
  }
  return lo;
}

__global__ void k_multi_prologue(MultiArgs m) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= m.total_points) return;
  const int it = find_item(m.offsets, m.n_items, p);
  prologue_point(m.args[it], p - m.offsets[it]);
}

__global__ void __launch_bounds__(kOrderThreads) k_multi_order_scan(MultiArgs m) {
  const LaunchArgs& a = m.args[blockIdx.x];
  if (a.order_hist) order_scan(a);
}

__global__ void k_multi_order_scatter(MultiArgs m) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= m.total_points) return;
  const int it = find_item(m.offsets, m.n_items, p);
  if (m.args[it].order_hist) order_scatter(m.args[it], p - m.offsets[it]);
}

// thread per (global point, detector, component): TaylorF2 mixed items, two
// components, at most kMultiMaxDet detectors
__global__ void k_multi_reduce(MultiArgs m) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= m.total_points * kMultiMaxDet * 2) return;
  const int64_t p = idx % m.total_points, r = idx / m.total_points;
  const int d = (int)(r / 2), t = (int)(r % 2);
  const int it = find_item(m.offsets, m.n_items, p);
  const LaunchArgs& a = m.args[it];
  if (d < a.n_det && t < part_components(a)) reduce_chain(a, p - m.offsets[it], d, t);
}

__global__ void k_multi_finalize(MultiArgs m) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= m.total_points) return;
  const int it = find_item(m.offsets, m.n_items, p);
  finalize_point(m.args[it], p - m.offsets[it], 1);
}

// Persistent: each CTA pulls work units of kernel class q = 2 D + CPLX
// (analyses with D detectors and that partial-sum kind; units
// [unit_begin[q], unit_begin[q + 1])) until none is left.  Every unit covers at
// most kChunksPerGroup chunks, so units of short and long analyses cost about
// the same.  One kernel per class keeps the register allocation of the
// single-analysis kernel.
template <int D, bool CPLX>
__global__ void __launch_bounds__(kPointsPerCta, 5) k_multi_tf2(MultiArgs m) {
  constexpr int q = 2 * D + (CPLX ? 1 : 0);
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ uint64_t bar[2];
  __shared__ unsigned long long s_kmax;
  __shared__ int64_t s_unit;
  if (threadIdx.x == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    mbar_fence_init();
  }
  int64_t it_global = 0;
  uint2* s_w = reinterpret_cast<uint2*>(smem);
  const int64_t ub = m.unit_begin[q], ue = m.unit_begin[q + 1];
  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) s_unit = ub + atomicAdd(m.counter + q, 1);
    __syncthreads();
    const int64_t u = s_unit;
    if (u >= ue) break;
    const int4 wu = m.units[u];
    const LaunchArgs& a = m.args[wu.x];
    tf2_unit<D, CPLX>(a, wu.y, wu.z, s_w, bar, &s_kmax, it_global, a.rf_count ? *a.rf_count : 0);
  }
}

// Accurate variant for the items of class (D, CPLX): the warps of the grid
// take the (marked point, group) units of each item in turn, continuing the
// round-robin from item to item.
template <int D, bool CPLX>
__global__ void __launch_bounds__(kAccThreads) k_multi_tf2_acc(MultiArgs m) {
  __shared__ float4 tab[kCosTable];
  const int wpc = kAccThreads / 32;
  const int64_t nw = (int64_t)gridDim.x * wpc, w = (int64_t)blockIdx.x * wpc + (threadIdx.x >> 5);
  bool loaded = false;
  int64_t base = 0;  // units of the earlier items of the class
  for (int it = 0; it < m.n_items; ++it) {
    const LaunchArgs& a = m.args[it];
    if (a.n_det != D || (a.cplx != 0) != CPLX || !a.rf_count || !(a.rf_tol > 0)) continue;
    const int64_t units = (int64_t)*a.rf_count * a.n_groups;
    if (units == 0) continue;
    if (!loaded) {  // uniform over the CTA: every thread sees the same items and counts
      load_cos_table(tab, a.cos_tab);
      __syncthreads();
      loaded = true;
    }
    for (int64_t u = ((w - base) % nw + nw) % nw; u < units; u += nw)
      acc_unit<D, CPLX>(a, a.order[u / a.n_groups], u % a.n_groups, tab);
    base += units;
  }
}

template <int D, bool CPLX, bool ACC>
static int ctas_per_sm_d() {
  static int n = 0;
  if (n == 0) {
    if (ACC) {
      if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_multi_tf2_acc<D, CPLX>, kAccThreads, 0) != cudaSuccess ||
          n < 1)
        n = 1;
      return n;
    }
    const int smem = 2 * D * kChunkMixed * 8;
    if (cudaFuncSetAttribute(k_multi_tf2<D, CPLX>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess)
      return 1;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_multi_tf2<D, CPLX>, kPointsPerCta, smem) != cudaSuccess ||
        n < 1)
      n = 1;
  }
  return n;
}

int multi_tf2_ctas_per_sm(int q, bool acc) {
  switch (q) {
    case 2: return acc ? ctas_per_sm_d<1, false, true>() : ctas_per_sm_d<1, false, false>();
    case 3: return acc ? ctas_per_sm_d<1, true, true>() : ctas_per_sm_d<1, true, false>();
    case 4: return acc ? ctas_per_sm_d<2, false, true>() : ctas_per_sm_d<2, false, false>();
    case 5: return acc ? ctas_per_sm_d<2, true, true>() : ctas_per_sm_d<2, true, false>();
    case 6: return acc ? ctas_per_sm_d<3, false, true>() : ctas_per_sm_d<3, false, false>();
    default: return acc ? ctas_per_sm_d<3, true, true>() : ctas_per_sm_d<3, true, false>();
  }
}

cudaError_t side_stream_create(SideStream* side) {
  int least = 0, greatest = 0;
  cudaError_t e = cudaDeviceGetStreamPriorityRange(&least, &greatest);
  if (e != cudaSuccess) return e;
  if ((e = cudaStreamCreateWithPriority(&side->stream, cudaStreamNonBlocking, greatest)) != cudaSuccess) return e;
  if ((e = cudaEventCreateWithFlags(&side->fork, cudaEventDisableTiming)) != cudaSuccess) return e;
  return cudaEventCreateWithFlags(&side->join, cudaEventDisableTiming);
}

void side_stream_destroy(SideStream* side) {
  if (side->stream) cudaStreamSynchronize(side->stream);
  if (side->fork) cudaEventDestroy(side->fork);
  if (side->join) cudaEventDestroy(side->join);
  if (side->stream) cudaStreamDestroy(side->stream);
  *side = SideStream();
}

cudaError_t side_fork(SideStream& side, cudaStream_t s) {
  cudaError_t e = cudaEventRecord(side.fork, s);
  if (e != cudaSuccess) return e;
  return cudaStreamWaitEvent(side.stream, side.fork, 0);
}

cudaError_t side_join(SideStream& side, cudaStream_t s) {
  cudaError_t e = cudaEventRecord(side.join, side.stream);
  if (e != cudaSuccess) return e;
  return cudaStreamWaitEvent(s, side.join, 0);
}

cudaError_t launch_multi(const MultiArgs& m, const int* ctas, const int* ctas_acc, cudaStream_t s, SideStream* side) {
  const int threads = kPointThreads;
  const unsigned pblocks = (unsigned)((m.total_points + threads - 1) / threads);
  k_multi_prologue<<<pblocks, threads, 0, s>>>(m);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  if (m.ordered) {
    k_multi_order_scan<<<(unsigned)m.n_items, kOrderThreads, 0, s>>>(m);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    k_multi_order_scatter<<<(unsigned)((m.total_points + 127) / 128), 128, 0, s>>>(m);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  // the accurate kernels on the side stream, beside the fast ones
  bool any_acc = false;
  for (int q = 2; q < kMultiClasses; ++q) any_acc = any_acc || ctas_acc[q] > 0;
  cudaStream_t sa = any_acc && side ? side->stream : s;
  if (any_acc && side && (e = side_fork(*side, s)) != cudaSuccess) return e;
  for (int q = 2; q < kMultiClasses; ++q) {
    if (ctas_acc[q] <= 0) continue;
    const unsigned ga = (unsigned)ctas_acc[q];
    switch (q) {
      case 2: k_multi_tf2_acc<1, false><<<ga, kAccThreads, 0, sa>>>(m); break;
      case 3: k_multi_tf2_acc<1, true><<<ga, kAccThreads, 0, sa>>>(m); break;
      case 4: k_multi_tf2_acc<2, false><<<ga, kAccThreads, 0, sa>>>(m); break;
      case 5: k_multi_tf2_acc<2, true><<<ga, kAccThreads, 0, sa>>>(m); break;
      case 6: k_multi_tf2_acc<3, false><<<ga, kAccThreads, 0, sa>>>(m); break;
      default: k_multi_tf2_acc<3, true><<<ga, kAccThreads, 0, sa>>>(m); break;
    }
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  for (int q = 2; q < kMultiClasses; ++q) {
    if (ctas[q] <= 0) continue;
    const int smem = 2 * (q / 2) * kChunkMixed * 8;
    const unsigned g = (unsigned)ctas[q];
    switch (q) {
      case 2: k_multi_tf2<1, false><<<g, kPointsPerCta, smem, s>>>(m); break;
      case 3: k_multi_tf2<1, true><<<g, kPointsPerCta, smem, s>>>(m); break;
      case 4: k_multi_tf2<2, false><<<g, kPointsPerCta, smem, s>>>(m); break;
      case 5: k_multi_tf2<2, true><<<g, kPointsPerCta, smem, s>>>(m); break;
      case 6: k_multi_tf2<3, false><<<g, kPointsPerCta, smem, s>>>(m); break;
      default: k_multi_tf2<3, true><<<g, kPointsPerCta, smem, s>>>(m); break;
    }
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  if (any_acc && side && (e = side_join(*side, s)) != cudaSuccess) return e;
  const int64_t chains = m.total_points * kMultiMaxDet * 2;
  k_multi_reduce<<<(unsigned)((chains + 127) / 128), 128, 0, s>>>(m);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  k_multi_finalize<<<pblocks, threads, 0, s>>>(m);
  return cudaGetLastError();
}

}  // namespace gwl
