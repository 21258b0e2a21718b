// Host+device float64 math used by the finalize step: ln I0 and the bicubic
// B-spline of the distance-marginalisation table.  Compiled for both sides so
// that the CPU tests can check it through gwl_host_math() without a GPU.
#pragma once

#include <cmath>

namespace gwl {

// ln I0(|x|) = log(i0e(x)) + |x| (bilby/gw/utils.py:1006-1022).
// Below 500 the library Bessel function is exact enough and cannot overflow;
// above, the large-argument expansion
//   I0(x) = e^x / sqrt(2 pi x) * sum_k ((2k-1)!!)^2 / (k! 8^k x^k)
// (Abramowitz & Stegun 9.7.1) converges to double precision in a few terms.
__host__ __device__ inline double ln_i0(double x) {
  x = fabs(x);
  if (x < 500.0) {
#ifdef __CUDA_ARCH__
    return log(cyl_bessel_i0(x));
#else
    return std::log(std::cyl_bessel_i(0.0, x));
#endif
  }
  const double inv = 1.0 / (8.0 * x);
  double term = 1.0, sum = 1.0;
  for (int k = 1; k < 12; ++k) {
    const double odd = 2.0 * k - 1.0;
    term *= odd * odd * inv / k;
    sum += term;
  }
  return x - 0.5 * log(6.283185307179586 * x) + log(sum);
}

// Cox-de Boor values of the k+1 non-zero B-splines at x on knot interval
// [t[L], t[L+1]) (the recurrence of FITPACK's fpbspl, as used by scipy's
// RectBivariateSpline.__call__ -> bispev).
__host__ __device__ inline void bspline_values(const double* t, int k, double x, int L, double* h) {
  double hh[4];
  h[0] = 1.0;
  for (int j = 1; j <= k; ++j) {
    for (int i = 0; i < j; ++i) hh[i] = h[i];
    h[0] = 0.0;
    for (int i = 1; i <= j; ++i) {
      const int li = L + i;
      const int lj = li - j;
      if (t[li] == t[lj]) {
        h[i] = 0.0;
      } else {
        const double f = hh[i - 1] / (t[li] - t[lj]);
        h[i - 1] += f * (t[li] - x);
        h[i] = f * (x - t[lj]);
      }
    }
  }
}

// Knot interval for x on a knot vector of length n with degree k, with
// x clamped to [t[k], t[n-k-1]] (fpbisp).
__host__ __device__ inline int bspline_interval(const double* t, int n, int k, double& x) {
  const double tb = t[k], te = t[n - k - 1];
  if (x < tb) x = tb;
  if (x > te) x = te;
  int lo = k, hi = n - k - 2;  // largest L in [k, n-k-2] with t[L] <= x
  while (lo < hi) {
    const int mid = (lo + hi + 1) / 2;
    if (t[mid] <= x) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// Bicubic spline value at (x, y); -inf outside the bounding box
// (BoundedRectBivariateSpline, bilby/core/utils/calculus.py:221-262).
__host__ __device__ inline double bicubic_eval(const double* tx, int nx, const double* ty, int ny, const double* c,
                                               const double* bbox, double x, double y) {
  if (!(x >= bbox[0] && x <= bbox[1] && y >= bbox[2] && y <= bbox[3])) return -INFINITY;
  const int Lx = bspline_interval(tx, nx, 3, x);
  const int Ly = bspline_interval(ty, ny, 3, y);
  double hx[4], hy[4];
  bspline_values(tx, 3, x, Lx, hx);
  bspline_values(ty, 3, y, Ly, hy);
  const int ncy = ny - 4;
  double s = 0.0;
  for (int i = 0; i < 4; ++i) {
    const double* row = c + (size_t)(Lx - 3 + i) * ncy + (Ly - 3);
    double r = 0.0;
    for (int j = 0; j < 4; ++j) r += row[j] * hy[j];
    s += r * hx[i];
  }
  return s;
}

// ln I0(x) - x for x >= 0 in float32 (the large part x is added in float64
// by the caller): the library Bessel function below 80, the large-argument
// expansion (A&S 9.7.1) above.
__device__ inline float ln_i0_minus_x(float x) {
  if (x < 80.0f) return logf(cyl_bessel_i0f(x)) - x;
  const float inv = 1.0f / (8.0f * x);
  const float sum = 1.0f + inv * (1.0f + inv * (4.5f + inv * 37.5f));
  return -0.5f * logf(6.2831853f * x) + logf(sum);
}

__device__ inline void bspline_values_f(const float* t, int k, float x, int L, float* h) {
  float hh[4];
  h[0] = 1.0f;
  for (int j = 1; j <= k; ++j) {
    for (int i = 0; i < j; ++i) hh[i] = h[i];
    h[0] = 0.0f;
    for (int i = 1; i <= j; ++i) {
      const int li = L + i;
      const int lj = li - j;
      if (t[li] == t[lj]) {
        h[i] = 0.0f;
      } else {
        const float f = hh[i - 1] / (t[li] - t[lj]);
        h[i - 1] += f * (t[li] - x);
        h[i] = f * (x - t[lj]);
      }
    }
  }
}

__device__ inline int bspline_interval_f(const float* t, int n, int k, float& x) {
  const float tb = t[k], te = t[n - k - 1];
  if (x < tb) x = tb;
  if (x > te) x = te;
  int lo = k, hi = n - k - 2;
  while (lo < hi) {
    const int mid = (lo + hi + 1) / 2;
    if (t[mid] <= x) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// float32 copy of bicubic_eval (same knots and coefficients rounded to float)
__device__ inline float bicubic_eval_f(const float* tx, int nx, const float* ty, int ny, const float* c,
                                       const double* bbox, float x, float y) {
  if (!((double)x >= bbox[0] && (double)x <= bbox[1] && (double)y >= bbox[2] && (double)y <= bbox[3]))
    return -INFINITY;
  const int Lx = bspline_interval_f(tx, nx, 3, x);
  const int Ly = bspline_interval_f(ty, ny, 3, y);
  float hx[4], hy[4];
  bspline_values_f(tx, 3, x, Lx, hx);
  bspline_values_f(ty, 3, y, Ly, hy);
  const int ncy = ny - 4;
  float s = 0.0f;
  for (int i = 0; i < 4; ++i) {
    const float* row = c + (size_t)(Lx - 3 + i) * ncy + (Ly - 3);
    float r = 0.0f;
    for (int j = 0; j < 4; ++j) r += row[j] * hy[j];
    s += r * hx[i];
  }
  return s;
}

// bicubic_eval_f split for many x at one y: the y-axis interval and B-spline
// values once (SplineRowF), then per x the same interval search, values and
// sums in the same order (the <d|h> axis is log-spaced, so the search stays).
struct SplineRowF {
  int Ly;
  int inside;  // y within the table's bounding box
  float hy[4];
};

__device__ inline SplineRowF bicubic_row_f(const float* ty, int ny, const double* bbox, float y) {
  SplineRowF row;
  row.inside = (double)y >= bbox[2] && (double)y <= bbox[3];
  row.Ly = 3;
  row.hy[0] = row.hy[1] = row.hy[2] = row.hy[3] = 0.f;
  if (row.inside) {
    row.Ly = bspline_interval_f(ty, ny, 3, y);
    bspline_values_f(ty, 3, y, row.Ly, row.hy);
  }
  return row;
}

// ... with the table's x bounds as float32 (bx[0] = bbox[0] rounded up,
// bx[1] = bbox[1] rounded down, so that the test of a float32 x is the same
// as against the float64 bounds, without float64 arithmetic)
__device__ inline float bicubic_eval_row_ff(const float* tx, int nx, int ny, const float* c, const float* bx, float x,
                                            const SplineRowF& row);

__device__ inline float bicubic_eval_row_f(const float* tx, int nx, int ny, const float* c, const double* bbox,
                                           float x, const SplineRowF& row) {
  if (!((double)x >= bbox[0] && (double)x <= bbox[1] && row.inside)) return -INFINITY;
  const int Lx = bspline_interval_f(tx, nx, 3, x);
  float hx[4];
  bspline_values_f(tx, 3, x, Lx, hx);
  const int ncy = ny - 4;
  float s = 0.0f;
  for (int i = 0; i < 4; ++i) {
    const float* rowc = c + (size_t)(Lx - 3 + i) * ncy + (row.Ly - 3);
    float r = 0.0f;
    for (int j = 0; j < 4; ++j) r += rowc[j] * row.hy[j];
    s += r * hx[i];
  }
  return s;
}

__device__ inline float bicubic_eval_row_ff(const float* tx, int nx, int ny, const float* c, const float* bx, float x,
                                            const SplineRowF& row) {
  if (!(x >= bx[0] && x <= bx[1] && row.inside)) return -INFINITY;
  const int Lx = bspline_interval_f(tx, nx, 3, x);
  float hx[4];
  bspline_values_f(tx, 3, x, Lx, hx);
  const int ncy = ny - 4;
  float s = 0.0f;
  for (int i = 0; i < 4; ++i) {
    const float* rowc = c + (size_t)(Lx - 3 + i) * ncy + (row.Ly - 3);
    float r = 0.0f;
    for (int j = 0; j < 4; ++j) r += rowc[j] * row.hy[j];
    s += r * hx[i];
  }
  return s;
}

}  // namespace gwl
