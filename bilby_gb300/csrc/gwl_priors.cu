// Prior rescaling and parameter conversion on the device: unit-cube samples
// to the [GWL_NPARAM][B] parameter block in one launch, one thread per point.
// The inverse CDFs follow bilby/core/prior/analytical.py (Uniform 214-225,
// PowerLaw / LogUniform 107-130, Cosine 415-421, Sine 475-481, Gaussian
// 535-545, TruncatedGaussian 627-634), interpolated.py:88-94 with scipy's
// linear interp1d (Interped, AlignedSpin) and bilby/gw/prior.py:401-446
// (UniformInComponentsMassRatio: a cubic interpolating spline of the inverse
// CDF); the conversions follow bilby/gw/conversion.py:849-990 (chirp mass,
// total mass and mass ratio to component masses) and the cos_theta_jn rule
// of convert_to_lal_binary_black_hole_parameters.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "gwl_device.cuh"
#include "gwl_internal.h"
#include "gwl_math.cuh"

namespace gwl {
// detector-frame conversion of a prior program (gwl_priors_set_frame)
struct PriorFrame {
  int has_rotation = 0, has_vertex = 0;
  double rotation[9] = {};
  double vertex[3] = {};
};
}  // namespace gwl

struct gwl_priors {
  int n = 0;
  gwl::PriorEntry* d_entries = nullptr;
  std::vector<double*> tables;
  gwl::PriorFrame frame;
  std::mutex mu;
};

namespace gwl {

__device__ __forceinline__ double table_linear(const PriorEntry& e, double u) {
  // scipy interp1d (linear): first x >= u, clipped to [1, n - 1]
  const int n = e.table_n;
  int lo = 0, hi = n;
  while (lo < hi) {
    const int mid = (lo + hi) / 2;
    if (e.x[mid] < u) lo = mid + 1; else hi = mid;
  }
  const int j = lo < 1 ? 1 : (lo > n - 1 ? n - 1 : lo);
  const double xl = e.x[j - 1], xh = e.x[j], yl = e.y[j - 1], yh = e.y[j];
  return (yh - yl) / (xh - xl) * (u - xl) + yl;
}

__device__ __forceinline__ double table_bspline(const PriorEntry& e, double u) {
  if (e.p[2] != 0.0) u = 2.0 * fmin(u, 1.0 - u);  // equal-mass folding (arXiv:2111.13619 App. A)
  const int nk = e.table_n;                        // knots; coefficients nk - 4
  if (u < e.x[3]) return e.p[0];
  if (u > e.p[3]) return e.p[1];
  double x = u;
  const int L = bspline_interval(e.x, nk, 3, x);
  double h[4];
  bspline_values(e.x, 3, x, L, h);
  double s = 0.0;
  for (int q = 0; q < 4; ++q) s += e.y[L - 3 + q] * h[q];
  return s;
}

__device__ __forceinline__ double prior_value(const PriorEntry& e, double u) {
  switch (e.kind) {
    case GWL_PRIOR_DELTA: return e.p[0];
    case GWL_PRIOR_UNIFORM: return e.p[0] + u * (e.p[1] - e.p[0]);
    case GWL_PRIOR_POWERLAW: {
      const double al = e.p[0], a = e.p[1], b = e.p[2];
      if (al == -1.0) return a * exp(u * log(b / a));
      return pow(pow(a, 1.0 + al) + u * (pow(b, 1.0 + al) - pow(a, 1.0 + al)), 1.0 / (1.0 + al));
    }
    case GWL_PRIOR_SINE: {
      const double norm = 1.0 / (cos(e.p[0]) - cos(e.p[1]));
      return acos(cos(e.p[0]) - u / norm);
    }
    case GWL_PRIOR_COSINE: {
      const double norm = 1.0 / (sin(e.p[1]) - sin(e.p[0]));
      return asin(u / norm + sin(e.p[0]));
    }
    case GWL_PRIOR_GAUSSIAN: return e.p[0] + erfinv(2.0 * u - 1.0) * 1.4142135623730951 * e.p[1];
    case GWL_PRIOR_TRUNCATED_GAUSSIAN:
      return erfinv(2.0 * u * e.p[3] + erf((e.p[2] - e.p[0]) / 1.4142135623730951 / e.p[1])) *
                 1.4142135623730951 * e.p[1] + e.p[0];
    case GWL_PRIOR_TABLE_LINEAR: return table_linear(e, u);
    case GWL_PRIOR_TABLE_BSPLINE: return table_bspline(e, u);
    default: return NAN;
  }
}

__global__ void k_priors(const PriorEntry* entries, int n, const double* unit, int64_t B, double* params,
                         PriorFrame frame) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= B) return;
  double mc = NAN, q = NAN, mt = NAN, cti = NAN, zen = NAN, azi = NAN, tdet = NAN;
  bool has_mc = false, has_q = false, has_mt = false, has_cti = false, has_zen = false, has_azi = false,
       has_tdet = false;
  for (int k = 0; k < n; ++k) {
    const PriorEntry& e = entries[k];
    const double u = e.column >= 0 ? unit[(int64_t)e.column * B + i] : 0.0;
    const double v = prior_value(e, u);
    switch (e.target) {
      case GWL_T_CHIRP_MASS: mc = v; has_mc = true; break;
      case GWL_T_MASS_RATIO: q = v; has_q = true; break;
      case GWL_T_TOTAL_MASS: mt = v; has_mt = true; break;
      case GWL_T_COS_THETA_JN: cti = v; has_cti = true; break;
      case GWL_T_ZENITH: zen = v; has_zen = true; break;
      case GWL_T_AZIMUTH: azi = v; has_azi = true; break;
      case GWL_T_DETECTOR_TIME: tdet = v; has_tdet = true; break;
      default:
        if (e.target >= 0 && e.target < GWL_NPARAM) params[(int64_t)e.target * B + i] = v;
    }
  }
  if (has_q && (has_mc || has_mt)) {
    // conversion.py:969-990, 849-870
    const double total = has_mt ? mt : mc * pow(1.0 + q, 1.2) / pow(q, 0.6);
    const double m1 = total / (1.0 + q);
    params[(int64_t)GWL_P_MASS_1 * B + i] = m1;
    params[(int64_t)GWL_P_MASS_2 * B + i] = m1 * q;
  }
  if (has_cti) params[(int64_t)GWL_P_THETA_JN * B + i] = acos(cti);
  // base.py:1091-1137: the sampled time is the reference detector's when it
  // is sampled, else geocent_time
  const double t = has_tdet ? tdet : params[(int64_t)GWL_P_GEOCENT_TIME * B + i];
  if (frame.has_rotation && has_zen && has_azi) {
    // zenith / azimuth in the detector-pair frame to ra / dec (gw/utils.py:232-256)
    const double wx = sin(zen) * cos(azi), wy = sin(zen) * sin(azi), wz = cos(zen);
    const double* R = frame.rotation;
    const double ox = R[0] * wx + R[1] * wy + R[2] * wz;
    const double oy = R[3] * wx + R[4] * wy + R[5] * wz;
    const double oz = R[6] * wx + R[7] * wy + R[8] * wz;
    const double theta = acos(oz);
    const double phi = pymod(atan2(oy, ox), kTwoPi);
    params[(int64_t)GWL_P_RA * B + i] = pymod(phi + gmst_radians(t), kTwoPi);
    params[(int64_t)GWL_P_DEC * B + i] = kPi / 2 - theta;
  }
  if (frame.has_vertex && has_tdet) {
    // geometry.py:319-343: geocent_time = t - time_delay_from_geocenter(vertex, ra, dec, t)
    const double ra = params[(int64_t)GWL_P_RA * B + i], dec = params[(int64_t)GWL_P_DEC * B + i];
    const double gmst = pymod(gmst_radians(t), kTwoPi);
    const double ph = ra - gmst, th = kPi / 2 - dec;
    const double ox = sin(th) * cos(ph), oy = sin(th) * sin(ph), oz = cos(th);
    const double delay = ((0.0 - frame.vertex[0]) * ox + (0.0 - frame.vertex[1]) * oy + (0.0 - frame.vertex[2]) * oz) /
                         kSpeedOfLight;
    params[(int64_t)GWL_P_GEOCENT_TIME * B + i] = t - delay;
  }
}

}  // namespace gwl

using gwl::set_error;

extern "C" {

int gwl_priors_create(const gwl_prior* entries, int32_t n, gwl_priors** out) {
  if (!out || n < 0 || (n > 0 && !entries)) {
    set_error("gwl_priors_create: null argument");
    return GWL_ERR_ARGUMENT;
  }
  auto* p = new gwl_priors();
  std::vector<gwl::PriorEntry> dev(n);
  for (int k = 0; k < n; ++k) {
    const gwl_prior& e = entries[k];
    gwl::PriorEntry& d = dev[k];
    std::memset(&d, 0, sizeof(d));
    d.kind = e.kind;
    d.target = e.target;
    d.column = e.column;
    d.table_n = e.table_n;
    for (int q = 0; q < 4; ++q) d.p[q] = e.p[q];
    const bool table = e.kind == GWL_PRIOR_TABLE_LINEAR || e.kind == GWL_PRIOR_TABLE_BSPLINE;
    if (e.kind < GWL_PRIOR_DELTA || e.kind > GWL_PRIOR_TABLE_BSPLINE ||
        (e.target < 0 || (e.target >= GWL_NPARAM && (e.target < GWL_T_CHIRP_MASS || e.target > GWL_T_DETECTOR_TIME)))) {
      set_error("gwl_priors_create: unknown prior kind or target in entry " + std::to_string(k));
      gwl_priors_destroy(p);
      return GWL_ERR_ARGUMENT;
    }
    if (table) {
      const int need = e.kind == GWL_PRIOR_TABLE_BSPLINE ? 8 : 2;
      if (e.table_n < need || !e.table_x || !e.table_y) {
        set_error("gwl_priors_create: table too short in entry " + std::to_string(k));
        gwl_priors_destroy(p);
        return GWL_ERR_ARGUMENT;
      }
      const int ny = e.kind == GWL_PRIOR_TABLE_BSPLINE ? e.table_n - 4 : e.table_n;
      double *dx = nullptr, *dy = nullptr;
      if (cudaMalloc(&dx, sizeof(double) * e.table_n) != cudaSuccess ||
          cudaMalloc(&dy, sizeof(double) * ny) != cudaSuccess) {
        cudaFree(dx);
        set_error("gwl_priors_create: cudaMalloc failed");
        gwl_priors_destroy(p);
        return GWL_ERR_MEMORY;
      }
      p->tables.push_back(dx);
      p->tables.push_back(dy);
      if (cudaMemcpy(dx, e.table_x, sizeof(double) * e.table_n, cudaMemcpyHostToDevice) != cudaSuccess ||
          cudaMemcpy(dy, e.table_y, sizeof(double) * ny, cudaMemcpyHostToDevice) != cudaSuccess) {
        set_error("gwl_priors_create: cudaMemcpy failed");
        gwl_priors_destroy(p);
        return GWL_ERR_CUDA;
      }
      d.x = dx;
      d.y = dy;
    }
  }
  if (n > 0) {
    if (cudaMalloc(&p->d_entries, sizeof(gwl::PriorEntry) * n) != cudaSuccess ||
        cudaMemcpy(p->d_entries, dev.data(), sizeof(gwl::PriorEntry) * n, cudaMemcpyHostToDevice) != cudaSuccess) {
      set_error("gwl_priors_create: device copy of the program failed");
      gwl_priors_destroy(p);
      return GWL_ERR_CUDA;
    }
  }
  p->n = n;
  *out = p;
  return GWL_OK;
}

int gwl_priors_destroy(gwl_priors* p) {
  if (!p) return GWL_OK;
  cudaFree(p->d_entries);
  for (double* t : p->tables) cudaFree(t);
  delete p;
  return GWL_OK;
}

int gwl_priors_rescale(gwl_priors* p, const double* unit, int64_t B, double* params, void* stream) {
  if (!p || B < 0 || (B > 0 && !params) || (B > 0 && p->n > 0 && !unit)) {
    set_error("gwl_priors_rescale: null argument");
    return GWL_ERR_ARGUMENT;
  }
  if (B == 0 || p->n == 0) return GWL_OK;
  std::lock_guard<std::mutex> g(p->mu);
  const int threads = 128;
  gwl::k_priors<<<(unsigned)((B + threads - 1) / threads), threads, 0, static_cast<cudaStream_t>(stream)>>>(
      p->d_entries, p->n, unit, B, params, p->frame);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error(std::string("gwl_priors_rescale: ") + cudaGetErrorString(e));
    return GWL_ERR_CUDA;
  }
  return GWL_OK;
}

int gwl_priors_set_frame(gwl_priors* p, const double* rotation, const double* vertex) {
  if (!p) {
    set_error("gwl_priors_set_frame: null argument");
    return GWL_ERR_ARGUMENT;
  }
  std::lock_guard<std::mutex> g(p->mu);
  p->frame.has_rotation = rotation ? 1 : 0;
  p->frame.has_vertex = vertex ? 1 : 0;
  for (int k = 0; k < 9; ++k) p->frame.rotation[k] = rotation ? rotation[k] : 0.0;
  for (int k = 0; k < 3; ++k) p->frame.vertex[k] = vertex ? vertex[k] : 0.0;
  return GWL_OK;
}

}  // extern "C"
