// Device helpers shared by the likelihood kernels.
//
// Per-point float64 prologue math (sidereal time, antenna patterns, geocentre
// time delay, TaylorF2 phase coefficients), float-float arithmetic used by the
// mixed-precision phase, and the bounded wait on a bulk-copy mbarrier.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "gwl_internal.h"

namespace gwl {

constexpr double kPi = 3.141592653589793;
constexpr double kTwoPi = 6.283185307179586;
constexpr double kSpeedOfLight = 299792458.0;
constexpr double kMtsunSI = 4.925490947641267e-06;  // G M_sun / c^3 (s)
constexpr double kPcSI = 3.085677581491367e16;      // parsec (m)
constexpr double kGammaE = 0.5772156649015329;

// GPS seconds at which each leap second was inserted (bilby/gw/time.py:74-93).
__constant__ double c_leap_seconds[18] = {
    46828800, 78364801, 109900802, 173059203, 252028804, 315187205, 346723206, 393984007, 425520008,
    457056009, 504489610, 551750411, 599184012, 820108813, 914803214, 1025136015, 1119744016, 1167264017};

// Greenwich mean sidereal time in radians, unreduced.  Same operation order
// as bilby/gw/time.py:114-165 (gps -> barebones UTC datetime -> Julian day ->
// t_hi / t_lo split), with explicit round-to-nearest ops so that the compiler
// does not contract the accumulation into FMAs.
__device__ __forceinline__ double gmst_radians(double gps) {
  const double gps_int = floor(gps);
  double nleap = 0.0;
#pragma unroll
  for (int i = 0; i < 18; ++i) nleap += (gps_int > c_leap_seconds[i]) ? 1.0 : 0.0;
  // 367*1980 - 7*(1980 + (1+9)//12)//4 + 275*1//9 + 6 = 723231 (time.py:57-66)
  const double second = __dsub_rn(gps_int, nleap);
  const double jd = __dadd_rn(__dadd_rn(723231.0, __ddiv_rn(second, 86400.0)), 1721013.5);
  const double t_hi = __ddiv_rn(__dsub_rn(jd, 2451545.0), 36525.0);
  const double t_lo = __ddiv_rn(__dsub_rn(gps, gps_int), 3155760000.0);
  const double t = __dadd_rn(t_hi, t_lo);
  double st = __dadd_rn(__dmul_rn(__dadd_rn(__dmul_rn(-6.2e-6, t), 0.093104), __dmul_rn(t, t)), 67310.54841);
  st = __dadd_rn(st, __dmul_rn(8640184.812866, t_lo));
  st = __dadd_rn(st, __dmul_rn(3155760000.0, t_lo));
  st = __dadd_rn(st, __dmul_rn(8640184.812866, t_hi));
  st = __dadd_rn(st, __dmul_rn(3155760000.0, t_hi));
  return __ddiv_rn(__dmul_rn(__dmul_rn(st, 2.0), kPi), 86400.0);
}

// Python's float modulo for a positive divisor.
__device__ __forceinline__ double pymod(double x, double y) {
  double r = fmod(x, y);
  if (r < 0) r += y;
  return r;
}

// Sines and cosines of the sky frame of one point (shared by its detectors).
struct SkyTrig {
  double sphi, cphi, sth, cth, sps, cps;
};

__device__ __forceinline__ SkyTrig sky_trig(double ra, double dec, double psi, double gmst_mod) {
  SkyTrig t;
  sincos(ra - gmst_mod, &t.sphi, &t.cphi);
  sincos(kPi / 2 - dec, &t.sth, &t.cth);
  sincos(psi, &t.sps, &t.cps);
  return t;
}

// Antenna patterns F+, Fx (bilby/gw/geometry.py:118-186 + 261-279) and the
// geocentre-to-detector delay (geometry.py:282-343) for one detector.
__device__ __forceinline__ void antenna_and_delay(const double* tensor, const double* vertex, const SkyTrig& t,
                                                  double* fplus, double* fcross, double* delay) {
  const double sphi = t.sphi, cphi = t.cphi, sth = t.sth, cth = t.cth, sps = t.sps, cps = t.cps;
  const double u[3] = {cphi * cth, cth * sphi, -sth};
  const double v[3] = {-sphi, cphi, 0.0};
  double m[3], n[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    m[i] = -u[i] * sps - v[i] * cps;
    n[i] = -u[i] * cps + v[i] * sps;
  }
  double fp = 0.0, fx = 0.0;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const double d = tensor[3 * i + j];
      fp += d * (m[i] * m[j] - n[i] * n[j]);
      fx += d * (m[i] * n[j] + n[i] * m[j]);
    }
  }
  *fplus = fp;
  *fcross = fx;
  const double om[3] = {sth * cphi, sth * sphi, cth};
  *delay = (om[0] * (0.0 - vertex[0]) + om[1] * (0.0 - vertex[1]) + om[2] * (0.0 - vertex[2])) / kSpeedOfLight;
}

__device__ __forceinline__ void antenna_and_delay(const double* tensor, const double* vertex, double ra,
                                                  double dec, double psi, double gmst_mod, double* fplus,
                                                  double* fcross, double* delay) {
  antenna_and_delay(tensor, vertex, sky_trig(ra, dec, psi, gmst_mod), fplus, fcross, delay);
}

// TaylorF2 phase coefficients a_k, l_k of
//   Psi(f) = -2 phase - pi/4 + 3/(128 eta v^5) sum_k (a_k + l_k ln v) v^k.
// Published PN coefficients: non-spinning 0..3.5PN from arXiv:0907.0700
// Eq. (3.18); aligned spin-orbit and spin-spin terms from arXiv:0810.5336,
// arXiv:1303.7412 and arXiv:1601.05588 (chi_s / chi_a form, kappa = 1).
__device__ __host__ inline void taylorf2_coefficients(double m1, double m2, double chi1, double chi2, double* a,
                                                      double* l) {
  const double m = m1 + m2;
  const double eta = m1 * m2 / (m * m);
  const double delta = (m1 - m2) / m;
  const double cs = 0.5 * (chi1 + chi2);
  const double ca = 0.5 * (chi1 - chi2);
  const double pi = 3.141592653589793;
  for (int k = 0; k < 8; ++k) {
    a[k] = 0.0;
    l[k] = 0.0;
  }
  a[0] = 1.0;
  a[2] = 3715.0 / 756.0 + 55.0 * eta / 9.0;
  a[3] = -16.0 * pi + 113.0 / 3.0 * delta * ca + (113.0 / 3.0 - 76.0 * eta / 3.0) * cs;
  a[4] = 15293365.0 / 508032.0 + 27145.0 * eta / 504.0 + 3085.0 * eta * eta / 72.0 +
         (-405.0 / 8.0 + 200.0 * eta) * ca * ca - 405.0 / 4.0 * delta * cs * ca +
         (-405.0 / 8.0 + 5.0 * eta / 2.0) * cs * cs;
  const double gamma = (732985.0 / 2268.0 - 24260.0 * eta / 81.0 - 340.0 * eta * eta / 9.0) * cs +
                       (732985.0 / 2268.0 + 140.0 * eta / 9.0) * delta * ca;
  const double c5 = pi * (38645.0 / 756.0 - 65.0 * eta / 9.0) - gamma;
  a[5] = c5;
  l[5] = 3.0 * c5;
  a[6] = 11583231236531.0 / 4694215680.0 - 640.0 * pi * pi / 3.0 - 6848.0 * kGammaE / 21.0 -
         6848.0 / 21.0 * 1.3862943611198906 /* ln 4 */ +
         eta * (-15737765635.0 / 3048192.0 + 2255.0 * pi * pi / 12.0) + 76055.0 * eta * eta / 1728.0 -
         127825.0 * eta * eta * eta / 1296.0 +
         pi * (2270.0 / 3.0 * delta * ca + (2270.0 / 3.0 - 520.0 * eta) * cs) +
         (75515.0 / 144.0 - 8225.0 * eta / 18.0) * delta * cs * ca +
         (75515.0 / 288.0 - 263245.0 * eta / 252.0 - 480.0 * eta * eta) * ca * ca +
         (75515.0 / 288.0 - 232415.0 * eta / 504.0 + 1255.0 * eta * eta / 9.0) * cs * cs;
  l[6] = -6848.0 / 21.0;
  a[7] = pi * (77096675.0 / 254016.0 + 378515.0 * eta / 1512.0 - 74045.0 * eta * eta / 756.0) +
         (-25150083775.0 / 3048192.0 + 10566655595.0 * eta / 762048.0 - 1042165.0 * eta * eta / 3024.0 +
          5345.0 * eta * eta * eta / 36.0) *
             cs +
         delta * (-25150083775.0 / 3048192.0 + 26804935.0 * eta / 6048.0 - 1985.0 * eta * eta / 48.0) * ca;
}

// ---------------------------------------------------------------------------
// float-float ("double-float") arithmetic: value = hi + lo, |lo| <= ulp(hi)/2.
// Dekker/Knuth error-free transformations with FMA (Muller et al., Handbook of
// Floating-Point Arithmetic, ch. 4-5).
// ---------------------------------------------------------------------------
struct ff {
  float hi, lo;
};

__device__ __forceinline__ ff ff_from_double(double x) {
  ff r;
  r.hi = __double2float_rn(x);
  r.lo = __double2float_rn(x - (double)r.hi);
  return r;
}

// s += a * b with a, b float-float; TwoProduct via FMA, TwoSum accumulation.
__device__ __forceinline__ void ff_mac(float& s_hi, float& s_lo, float a_hi, float a_lo, float b_hi, float b_lo) {
  const float p = __fmul_rn(a_hi, b_hi);
  float e = __fmaf_rn(a_hi, b_hi, -p);
  e = __fmaf_rn(a_hi, b_lo, e);
  e = __fmaf_rn(a_lo, b_hi, e);
  const float s = __fadd_rn(s_hi, p);
  const float bb = __fsub_rn(s, s_hi);
  const float err = __fadd_rn(__fsub_rn(s_hi, __fsub_rn(s, bb)), __fsub_rn(p, bb));
  s_lo = __fadd_rn(s_lo, __fadd_rn(err, e));
  s_hi = s;
}

// Kahan-compensated float32 accumulation: the running sum is s - c.
__device__ __forceinline__ void kahan_add(float& s, float& c, float x) {
  const float y = __fsub_rn(x, c);
  const float t = __fadd_rn(s, y);
  c = __fsub_rn(__fsub_rn(t, s), y);
  s = t;
}

// exp(-a (f + sign * f0)^2) for the sine-Gaussian, with the argument formed
// in float-float so that its rounding error does not grow with its size
// (an error proportional to the argument would be smooth in f and add up
// coherently over the Gaussian); the exponential is the float32 expf of the
// high word, corrected to first order by the low word.
__device__ __forceinline__ float gauss_ff(float f, float f0h, float f0l, float ah, float al, float sign) {
  const float b = sign * f0h;
  const float s = __fadd_rn(f, b);
  const float bb = __fsub_rn(s, f);
  float e = __fadd_rn(__fsub_rn(f, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  e = __fadd_rn(e, sign * f0l);
  const float hi = __fadd_rn(s, e);
  const float lo = __fsub_rn(e, __fsub_rn(hi, s));
  const float p = __fmul_rn(hi, hi);
  float pe = __fmaf_rn(hi, hi, -p);
  pe = __fmaf_rn(2.0f * hi, lo, pe);
  const float q = __fmul_rn(ah, p);
  float qe = __fmaf_rn(ah, p, -q);
  qe = __fmaf_rn(ah, pe, qe);
  qe = __fmaf_rn(al, p, qe);
  return expf(-q) * (1.0f - qe);
}

// ---------------------------------------------------------------------------
// 1-D bulk asynchronous copies global -> shared, completed on an mbarrier.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_fence_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
}

// Requires: dst, src 16-byte aligned; bytes a multiple of 16.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Checked builds (-DGWL_CHECK): the gathers and scatters whose indices come
// from host-built tables (scatter lists, bin maps, transform bins) test the
// index first; a failed test records kDevStatusIndex in the status word and
// the access is skipped, so that a bad table reads back as GWL_ERR_CHECK
// instead of touching memory out of bounds.  Ordinary builds compile the
// test away.
#ifdef GWL_CHECK
__device__ __forceinline__ bool index_ok(int64_t i, int64_t n, int* status) {
  if (i >= 0 && i < n) return true;
  if (status) atomicExch(status, kDevStatusIndex);
  return false;
}
#define GWL_INDEX_OK(i, n, status) ::gwl::index_ok((int64_t)(i), (int64_t)(n), (status))
#else
#define GWL_INDEX_OK(i, n, status) true
#endif

// Bounded wait: gives up after `limit` polls, records the failure in the
// device status word and returns false.  Each poll suspends for a
// hardware-defined time slice, so the limit bounds the wait to well under a
// second.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, int* status, uint32_t limit) {
  for (uint32_t it = 0; it < limit; ++it) {
    if (mbar_try_wait(bar, parity)) return true;
  }
  if (status) atomicExch(status, kDevStatusTimeout);
  return false;
}

}  // namespace gwl
