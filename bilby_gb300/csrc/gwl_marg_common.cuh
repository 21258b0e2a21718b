// Device helpers shared by the time-marginalised kernels (gwl_marg.cu: one
// CTA per point over a whole FFT; gwl_marg_window.cu: the windowed four-step
// transform): source polarisations, the geocent_time prior's density, the
// relative-binning edge ratios and the per-sample marginalised lnL
// (bilby/gw/likelihood/base.py:794-820, 1027-1035).
#pragma once

#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>

#include "gwl_device.cuh"
#include "gwl_internal.h"
#include "gwl_math.cuh"

namespace gwl {

// The density of a geocent_time prior other than Uniform at GPS time t
// (LaunchArgs::tm_prior): Lagrange interpolation through the four table nodes
// around t, shifted inwards at the ends of the table (the nodes lie inside the
// prior's support, so a time between a support edge and the first node is
// extrapolated by less than one node spacing); zero beyond.  t - t0 is exact
// (t0 and the nodes are multiples of a power-of-two step), so a sample on a
// node reads that node's density exactly.
__device__ __forceinline__ double tm_prior_density(const LaunchArgs& a, double t) {
  const double x = (t - a.tm_prior_t0) * a.tm_prior_inv_h;
  if (!(x >= -1.0 && x <= (double)a.tm_prior_n)) return 0.0;
  const int64_t g = max((int64_t)0, min((int64_t)floor(x) - 1, a.tm_prior_n - 4));
  const double u = x - (double)g, u1 = u - 1.0, u2 = u - 2.0, u3 = u - 3.0;
  const double* p = a.tm_prior + g;
  const double v = (p[3] * u * u1 * u2 - p[0] * u1 * u2 * u3) / 6.0 + (p[1] * u * u2 * u3 - p[2] * u * u1 * u3) / 2.0;
  return fmax(v, 0.0);
}

__device__ __forceinline__ float tm_prior_density_f(const LaunchArgs& a, double t) {
  const double x = (t - a.tm_prior_t0) * a.tm_prior_inv_h;
  if (!(x >= -1.0 && x <= (double)a.tm_prior_n)) return 0.f;
  const int64_t g = max((int64_t)0, min((int64_t)floor(x) - 1, a.tm_prior_n - 4));
  const float u = (float)(x - (double)g), u1 = u - 1.f, u2 = u - 2.f, u3 = u - 3.f;
  const float* p = a.tm_prior_f + g;
  const float v = (p[3] * u * u1 * u2 - p[0] * u1 * u2 * u3) * (1.f / 6.f) + (p[1] * u * u2 * u3 - p[2] * u * u1 * u3) * 0.5f;
  return fmaxf(v, 0.f);
}

template <bool MIXED>
struct TmTypes;
template <>
struct TmTypes<true> {
  using C = float2;
  using R = float;
};
template <>
struct TmTypes<false> {
  using C = double2;
  using R = double;
};

__device__ __forceinline__ uint32_t bit_reverse(uint32_t k, int log2n) { return __brev(k) >> (32 - log2n); }

// Multi-banding with the IFFT-FFT <h|h>: the odd-bin part of point i summed
// over the bands b >= 1 and the detectors (zero without it).
__device__ __forceinline__ double mb_fft_hh_total(const LaunchArgs& a, int64_t i) {
  double s = 0.0;
  if (a.mb_fft_hh)
    for (int b = 1; b < a.mb_bands; ++b)
      for (int d = 0; d < a.n_det; ++d) s += a.mb_fft_hh[((int64_t)b * a.n_det + d) * a.B + i];
  return s;
}

// float64 source polarisations of the plain kernels at one frequency.
__device__ __forceinline__ bool plain_pols(const LaunchArgs& a, const PointRec& r, double f, double2& hp, double2& hx) {
  if (a.model == GWL_MODEL_SINEGAUSSIAN) {
    const double pi2 = 9.869604401089358;
    const double fm = f - r.sg_f0, fpl = f + r.sg_f0;
    const double neg = exp(-(fm * fm) * pi2 * r.a[3]);
    const double pos = exp(-(fpl * fpl) * pi2 * r.a[3]);
    hp = make_double2(r.a[0] * (neg + pos) / r.a[1], 0.0);
    hx = make_double2(0.0, -(r.a[0] * (neg - pos) / r.a[2]));
    return true;
  }
  if (f < a.fmin || f >= r.f_isco) return false;
  const double v = cbrt(kPi * r.m_sec * f), lnv = log(v);
  double s = 0.0, vk = 1.0;
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    s = s + (r.a[q] + r.l[q] * lnv) * vk;
    vk = vk * v;
  }
  const double psi = (-2.0 * r.phase - kPi / 4) + 3.0 / (128.0 * r.eta) * s / (v * v * v * v * v);
  const double amp = r.amp * pow(f, -7.0 / 6.0);
  double sp, cp;
  sincos(psi, &sp, &cp);
  const double ere = amp * cp, eim = -amp * sp, ci = r.cos_i, pf = (1.0 + ci * ci) / 2.0;
  hp = make_double2(pf * ere, pf * eim);
  hx = make_double2(ci * eim, -ci * ere);
  return true;
}

// The same TaylorF2 polarisations from a power-table entry t = {f^(1/3),
// ln(f) / 3, f^(-5/3), f^(-7/6)}; u = (pi M)^(1/3), pu5 = 3 / (128 eta u^5).
__device__ __forceinline__ bool tf2_pols_t(const LaunchArgs& a, const PointRec& r, const double4& t, double f,
                                           double u, double lnu, double pu5, double2& hp, double2& hx) {
  if (f < a.fmin || f >= r.f_isco) return false;
  const double v = u * t.x, lnv = lnu + t.y;
  double s = r.a[7];
#pragma unroll
  for (int q = 6; q >= 0; --q) s = s * v + r.a[q];
  const double v5 = v * v * v * v * v;
  s = s + lnv * (r.l[5] + r.l[6] * v) * v5;
  const double psi = (-2.0 * r.phase - kPi / 4) + pu5 * s * t.z;
  const double amp = r.amp * t.w;
  double sp, cp;
  sincos(psi, &sp, &cp);
  const double ere = amp * cp, eim = -amp * sp, ci = r.cos_i, pf = (1.0 + ci * ci) / 2.0;
  hp = make_double2(pf * ere, pf * eim);
  hx = make_double2(ci * eim, -ci * ere);
  return true;
}

// ... at grid bin k of the per-bin power table
__device__ __forceinline__ bool tf2_pols_tab(const LaunchArgs& a, const PointRec& r, int64_t k, double f, double u,
                                             double lnu, double pu5, double2& hp, double2& hx) {
  if (f < a.fmin || f >= r.f_isco) return false;
  return tf2_pols_t(a, r, a.ftab[k], f, u, lnu, pu5, hp, hx);
}

// (c + i s) *= (rc + i rs)
__device__ __forceinline__ void tm_rotate(double& c, double& s, double rc, double rs) {
  const double t = c * rc - s * rs;
  s = c * rs + s * rc;
  c = t;
}


// Relative binning (relative.py:365-378): the ratios h_d(f_e) / h0_d(f_e) of
// point r at the bin edges, rat[d * nE + e], over the CTA's threads.
template <int D>
__device__ void relbin_edge_ratios(const LaunchArgs& a, const PointRec& r, double2* rat) {
  const int nE = a.rb_edges;
  const bool tf2 = a.model == GWL_MODEL_TAYLORF2;
  const double u = tf2 ? cbrt(kPi * r.m_sec) : 0.0, lnu = tf2 ? log(u) : 0.0;
  const double pu5 = tf2 ? 3.0 / (128.0 * r.eta) / (u * u * u * u * u) : 0.0;
  for (int e = threadIdx.x; e < nE; e += blockDim.x) {
    const double f = a.rb_freq[e];
    double2 hp = make_double2(0.0, 0.0), hx = make_double2(0.0, 0.0);
    const bool on = r.valid && (tf2 ? tf2_pols_tab(a, r, a.rb_index[e], f, u, lnu, pu5, hp, hx)
                                    : plain_pols(a, r, f, hp, hx));
#pragma unroll
    for (int d = 0; d < D; ++d) {
      double2 q = make_double2(0.0, 0.0);
      if (on) {
        // interferometer.py:341-362 at explicit frequencies (no mask)
        const double sre = hp.x * r.fp[d] + hx.x * r.fx[d], sim = hp.y * r.fp[d] + hx.y * r.fx[d];
        double sn, cs;
        sincos(2.0 * kPi * r.dt[d] * f, &sn, &cs);
        const double hre = sre * cs + sim * sn, him = sim * cs - sre * sn;
        const double2 g = a.rb_h0inv[d][e];
        q = make_double2(hre * g.x - him * g.y, hre * g.y + him * g.x);
      }
      rat[d * nE + e] = q;
    }
  }
}

// This thread's share of <h|h> from the summary data (relative.py:403-405):
// sum over its bins b of b0 |r0|^2 + 2 b1 Re(r0 conj(r1)).
template <int D>
__device__ double relbin_hh_part(const LaunchArgs& a, const double2* rat) {
  const int nE = a.rb_edges, nB = nE - 1;
  double hh = 0.0;
  for (int b = threadIdx.x; b < nB; b += blockDim.x) {
    const double width = a.rb_freq[b + 1] - a.rb_freq[b];
#pragma unroll
    for (int d = 0; d < D; ++d) {
      const double2 q0 = rat[d * nE + b], q1 = rat[d * nE + b + 1];
      const double r0r = (q1.x + q0.x) / 2, r0i = (q1.y + q0.y) / 2;
      const double r1r = (q1.x - q0.x) / width, r1i = (q1.y - q0.y) / width;
      const double* sd = a.rb_sum[d] + (size_t)b * 6;
      hh += sd[4] * (r0r * r0r + r0i * r0i) + 2.0 * sd[5] * (r0r * r1r + r0i * r1i);
    }
  }
  return hh;
}

// GPS time of FFT sample j: base.py:1027-1035 (linspace(0, T, L + 1)[1:], the
// last sample exactly T) or multiband.py:714-717 (arange(L) * delta_tc).
__device__ __forceinline__ double tm_sample_time(const LaunchArgs& a, int64_t j, int64_t L, double step, double jit) {
  const double lin = a.tm_first ? ((j + 1 == L) ? a.duration : (double)(j + 1) * step) : (double)j * step;
  return (a.start_time0 + lin) + jit;
}

// Whether sample time t is inside the prior's support, and its log prior
// weight (base.py:807, prior(t_j) delta_tc; a Uniform prior's constant is
// applied once to the total instead, so lw = 0 for it).
template <bool MIXED>
__device__ __forceinline__ bool tm_log_weight(const LaunchArgs& a, double t, double& lw) {
  lw = 0.0;
  if (!(t >= a.t_min && t <= a.t_max)) return false;
  if (a.tm_prior) {
    if constexpr (MIXED) {
      const float pw = tm_prior_density_f(a, t);
      if (!(pw > 0.f)) return false;
      lw = (double)__logf(pw);
    } else {
      const double pw = tm_prior_density(a, t);
      if (!(pw > 0.0)) return false;
      lw = log(pw);
    }
  }
  return true;
}

// The marginalised lnL of one time sample from <d|h>(t_j) = xr + i xi
// (base.py:775-792): distance table, ln I0 or the real part.
__device__ __forceinline__ double tm_lnl_fp64(const LaunchArgs& a, double xr, double xi, double hh, double hh_ref,
                                              double sr) {
  if (a.dist_marg) {
    const double dx = a.phase_marg ? sqrt(xr * xr + xi * xi) * sr : xr * sr;
    return bicubic_eval(a.tx, a.nx, a.ty, a.ny, a.tc, a.bbox, dx, hh_ref);
  }
  if (a.phase_marg) return ln_i0(sqrt(xr * xr + xi * xi)) - hh / 2;
  return xr - hh / 2;
}

// ... float32 per-sample work, the large terms combined in float64; the
// distance spline's knots (s_tx) and its row at this point's <h|h> (row) in
// shared memory
__device__ __forceinline__ double tm_lnl_mixed(const LaunchArgs& a, float xr, float xi, double hh, double sr,
                                               const float* s_tx, const SplineRowF& row) {
  if (a.dist_marg) {
    const float dx = a.phase_marg ? sqrtf(xr * xr + xi * xi) * (float)sr : xr * (float)sr;
    return (double)bicubic_eval_row_f(s_tx, a.nx, a.ny, a.tc_f, a.bbox, dx, row);
  }
  if (a.phase_marg) {
    const float ax = sqrtf(xr * xr + xi * xi);
    return ((double)ax + (double)ln_i0_minus_x(ax)) - hh / 2;
  }
  return (double)xr - hh / 2;
}

// One sample into a running logsumexp (m = maximum so far, acc = sum of
// exp(l - m)).
template <bool MIXED>
__device__ __forceinline__ void tm_lse_push(double l, double& m, double& acc) {
  if (l > m) {
    acc = isfinite(m) ? acc * (MIXED ? (double)__expf((float)(m - l)) : exp(m - l)) + 1.0 : 1.0;
    m = l;
  } else if (isfinite(l)) {
    acc += MIXED ? (double)__expf((float)(l - m)) : exp(l - m);
  }
}

// The largest sensitivity dl_j / d|X_j| of the per-sample lnL over a window
// whose largest |<d|h>(t_j)| is xpk: 1 for the real part and for ln I0
// (I1 / I0 < 1); with the distance table sr E[d_ref / d], which grows with |X|
// (the table is convex in its first argument), so its value at xpk.  It comes
// from a central difference of the float32 spline row of the point's <h|h>
// (knots in shared memory; the float64 table's dependent loads would stall the
// CTA), with a margin for the difference's rounding.  |dlnL| is at most this
// times the largest error of X over the window.
__device__ inline double tm_sensitivity(const LaunchArgs& a, double xpk, double sr, const float* s_tx,
                                        const SplineRowF& row) {
  if (!a.dist_marg) return 1.0;
  const float dx = (float)(xpk * sr), del = fmaxf(1e-3f * dx, 1e-2f), lo = fmaxf(dx - del, 0.f);
  const float up = bicubic_eval_row_f(s_tx, a.nx, a.ny, a.tc_f, a.bbox, dx + del, row);
  const float dn = bicubic_eval_row_f(s_tx, a.nx, a.ny, a.tc_f, a.bbox, lo, row);
  const double d = fabs((double)up - (double)dn) / ((double)(dx + del) - (double)lo);
  return fmin(sr * (1.25 * d + 5e-3), 1e6);  // an undefined difference gives 1e6
}

// exp(-2 pi i t / L) for t < L / 2 in float64 and float32, one pair of tables
// per (device, FFT length), kept for the life of the process (gwl_marg.cu).
struct TwiddleTables {
  double2* d64 = nullptr;
  float2* d32 = nullptr;
};
cudaError_t twiddles_for(int64_t L, TwiddleTables* out);

}  // namespace gwl
