// Float64 source-model and detector-response kernels that write h(f) out.
// Used for injections and for checking the source models on their own; the
// likelihood kernels never materialise h(f).
#include <cuda_runtime.h>

#include <cmath>

#include "gwl_device.cuh"
#include "gwl_internal.h"
#include "gwl_math.cuh"

namespace gwl {

__global__ void k_polarizations(int model, const double* freq, int64_t n, const double* p, double fmin,
                                double2* plus, double2* cross) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const double f = freq[k];
  if (model == GWL_MODEL_SINEGAUSSIAN) {
    // bilby/gw/source.py:1197-1207
    const double hrss = p[GWL_P_HRSS], Q = p[GWL_P_Q], f0 = p[GWL_P_FREQUENCY];
    const double tau = Q / (1.4142135623730951 * kPi * f0);
    const double temp = Q / (4.0 * 1.7724538509055159 * f0);
    const double fm = f - f0, fp = f + f0;
    const double pi2 = 9.869604401089358;
    const double neg = exp(-(fm * fm) * pi2 * (tau * tau));
    const double pos = exp(-(fp * fp) * pi2 * (tau * tau));
    const double pref = hrss * 1.7724538509055159 * tau / 2;
    plus[k] = make_double2(pref * (neg + pos) / sqrt(temp * (1 + exp(-Q * Q))), 0.0);
    cross[k] = make_double2(0.0, -(pref * (neg - pos) / sqrt(temp * (1 - exp(-Q * Q)))));
    return;
  }
  const double m1 = p[GWL_P_MASS_1], m2 = p[GWL_P_MASS_2];
  const double m = m1 + m2, m_sec = m * kMtsunSI, eta = m1 * m2 / (m * m);
  const double f_isco = 1.0 / (6.0 * sqrt(6.0) * kPi * m_sec);
  if (!(f >= fmin && f < f_isco)) {
    plus[k] = make_double2(0.0, 0.0);
    cross[k] = make_double2(0.0, 0.0);
    return;
  }
  double a[8], l[8];
  taylorf2_coefficients(m1, m2, p[GWL_P_CHI_1], p[GWL_P_CHI_2], a, l);
  const double v = cbrt(kPi * m_sec * f), lnv = log(v);
  double s = 0.0, vk = 1.0;
  for (int q = 0; q < 8; ++q) {
    s = s + (a[q] + l[q] * lnv) * vk;
    vk = vk * v;
  }
  const double psi = -2.0 * p[GWL_P_PHASE] - kPi / 4 + 3.0 / (128.0 * eta) * s / (v * v * v * v * v);
  const double mc_sec = pow(eta, 0.6) * m * kMtsunSI;
  const double amp = sqrt(5.0 / 24.0) * pow(kPi, -2.0 / 3.0) * pow(mc_sec, 5.0 / 6.0) * kSpeedOfLight /
                     (p[GWL_P_LUMINOSITY_DISTANCE] * 1e6 * kPcSI) * pow(f, -7.0 / 6.0);
  const double ci = cos(p[GWL_P_THETA_JN]);
  double sp, cp;
  sincos(psi, &sp, &cp);
  const double ere = amp * cp, eim = -amp * sp;
  plus[k] = make_double2(ere * (1.0 + ci * ci) / 2.0, eim * (1.0 + ci * ci) / 2.0);
  cross[k] = make_double2(ci * eim, -ci * ere);
}

__global__ void k_response(DetGeom g, const double* freq, int64_t n, const double2* plus, const double2* cross,
                           const double* p, double2* resp) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const double tgeo = p[GWL_P_GEOCENT_TIME];
  const double gmst = pymod(gmst_radians(tgeo), kTwoPi);
  double fp, fx, delay;
  antenna_and_delay(g.tensor, g.vertex, p[GWL_P_RA], p[GWL_P_DEC], p[GWL_P_PSI], gmst, &fp, &fx, &delay);
  const double dt = (tgeo - g.start_time) + delay;
  const double2 hp = plus[k], hx = cross[k];
  const double sre = hp.x * fp + hx.x * fx, sim = hp.y * fp + hx.y * fx;
  double sn, cs;
  sincos(2.0 * kPi * dt * freq[k], &sn, &cs);
  resp[k] = make_double2(sre * cs + sim * sn, sim * cs - sre * sn);
}

cudaError_t launch_source_polarizations(int model, const double* freq, int64_t n, const double* params, double fmin,
                                        double* plus, double* cross, cudaStream_t s) {
  const int threads = 256;
  k_polarizations<<<(unsigned)((n + threads - 1) / threads), threads, 0, s>>>(
      model, freq, n, params, fmin, reinterpret_cast<double2*>(plus), reinterpret_cast<double2*>(cross));
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  return cudaStreamSynchronize(s);
}

cudaError_t launch_detector_response(const DetGeom& g, const double* freq, int64_t n, const double* plus,
                                     const double* cross, const double* params, double* resp, cudaStream_t s) {
  const int threads = 256;
  k_response<<<(unsigned)((n + threads - 1) / threads), threads, 0, s>>>(
      g, freq, n, reinterpret_cast<const double2*>(plus), reinterpret_cast<const double2*>(cross), params,
      reinterpret_cast<double2*>(resp));
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  return cudaStreamSynchronize(s);
}

// ---------------------------------------------------------------------------
// distance-marginalisation lookup table (bilby/gw/likelihood/base.py:994-1018)
// ---------------------------------------------------------------------------
__global__ void k_ln_i0_grid(const double* dh_axis, int n_dh, const double* scaling, int n, double* out) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (int64_t)n_dh * n) return;
  const int j = (int)(idx / n), k = (int)(idx % n);
  out[idx] = ln_i0(fabs(dh_axis[j] * scaling[k]));
}

// One warp per table entry (ii over <h|h>, jj over <d|h>): a weighted
// logsumexp over the distance grid, in scipy's form (entries with zero weight
// excluded from the maximum), reduced with a fixed shuffle tree.
__global__ void k_distance_table(const double* dh_axis, int n_dh, const double* hh_axis, int n_hh,
                                 const double* scaling, const double* scaling2, const double* weight, int n,
                                 const double* lni0, double log_norm, double* table) {
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= (int64_t)n_dh * n_hh) return;
  const int ii = (int)(warp / n_dh), jj = (int)(warp % n_dh);
  const double dh = dh_axis[jj], hh = hh_axis[ii];
  double m = -INFINITY;
  for (int k = lane; k < n; k += 32) {
    if (weight[k] == 0.0) continue;
    const double a = (lni0 ? lni0[(int64_t)jj * n + k] : dh * scaling[k]) - hh * scaling2[k] / 2;
    m = fmax(m, a);
  }
  for (int off = 16; off > 0; off >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, off));
  double s = 0.0;
  if (isfinite(m)) {
    for (int k = lane; k < n; k += 32) {
      if (weight[k] == 0.0) continue;
      const double a = (lni0 ? lni0[(int64_t)jj * n + k] : dh * scaling[k]) - hh * scaling2[k] / 2;
      s += weight[k] * exp(a - m);
    }
  }
  for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
  if (lane == 0) table[(int64_t)ii * n_dh + jj] = (isfinite(m) ? log(s) + m : m) - log_norm;
}

cudaError_t launch_distance_table(const double* dh_axis, int n_dh, const double* hh_axis, int n_hh,
                                  const double* scaling, const double* scaling2, const double* weight, int n,
                                  double* lni0_work, int phase, double log_norm, double* table) {
  if (phase) {
    const int64_t total = (int64_t)n_dh * n;
    k_ln_i0_grid<<<(unsigned)((total + 255) / 256), 256>>>(dh_axis, n_dh, scaling, n, lni0_work);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  const int64_t warps = (int64_t)n_dh * n_hh;
  k_distance_table<<<(unsigned)((warps * 32 + 255) / 256), 256>>>(dh_axis, n_dh, hh_axis, n_hh, scaling, scaling2,
                                                                  weight, n, phase ? lni0_work : nullptr, log_norm,
                                                                  table);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  return cudaDeviceSynchronize();
}

// Self-test of the bounded bulk-copy wait used by the likelihood kernels: one
// thread arms an mbarrier for 16 bytes of transaction and issues no copy, so
// the phase can never complete; mbar_wait_bounded gives up after `limit`
// polls and records kDevStatusTimeout.  Nothing is in flight when the CTA
// returns.  `arrived` receives 1 if the wait (impossibly) completed.
__global__ void k_wait_selftest(uint32_t limit, int* status, int* arrived) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x != 0) return;
  mbar_init(&bar, 1);
  mbar_fence_init();
  mbar_expect_tx(&bar, 16);
  *arrived = mbar_wait_bounded(&bar, 0, status, limit) ? 1 : 0;
}

cudaError_t launch_wait_selftest(uint32_t limit, int* status, int* arrived, cudaStream_t s) {
  k_wait_selftest<<<1, 32, 0, s>>>(limit, status, arrived);
  return cudaGetLastError();
}

}  // namespace gwl
