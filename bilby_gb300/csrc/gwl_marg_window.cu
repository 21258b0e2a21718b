// Time marginalisation of the fast likelihoods by a windowed four-step
// transform: relative binning (bilby/gw/likelihood/relative.py:398-420) and
// multi-banding (multiband.py:714-726, 792-800), with phase (ln I0) and
// distance (bicubic table) marginalisation composed as in base.py:775-820.
//
// The likelihood reads the transform X[j] = sum_n z_n exp(-2 pi i n j / L) of
// the integrand z only at the few hundred samples j inside the geocent_time
// prior, while L is 2^18 - 2^19 for a 128 s segment.  With L = N1 N2 (N2 a
// power of two up to 2048, N1 = L / N2 carrying any odd factor of L) and
// n = n1 + N1 n2:
//   B_n1[k] = sum_n2 z[n1 + N1 n2] exp(-2 pi i n2 k / N2)     (column FFTs)
//   X[j]    = sum_n1 exp(-2 pi i n1 j / L) B_n1[j mod N2]     (window sums)
// One CTA per parameter point takes G columns at a time: it evaluates their
// integrand straight into the first radix-2 stages (in registers), runs the
// remaining stages in shared memory and adds the columns' terms to the
// window's accumulators.  Nothing of size L goes through global memory: per
// point the kernel reads the integrand's tables (shared by every point, so
// L2-resident) and writes one double.  Work per point: L/2 log2(N2)
// butterflies and n_win N1 window terms, against L/2 log2(L) butterflies for
// the whole transform.
//
// Mixed precision: float32 integrand, transform and compensated window sums;
// relative binning keeps the per-bin ratio coefficients and <h|h> in float64,
// multi-banding (TaylorF2) forms its banded values with the exact fixed-point
// phase of the non-marginalised mixed kernel.  The
// error bound of a point is s (kWinErrNorm ||z||_2 + kWinErrPeak max_j |X_j|),
// s the largest sensitivity dl_j / d|X_j| over the window; points over the
// tolerance are marked and recomputed by the float64 kernel.
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

constexpr int kWinThreads = 512;
constexpr int kWinWarps = kWinThreads / 32;
constexpr int kWinOutRows = 1024;   // mixed output twiddles: q = 1024 q1 + q2
// Error model of the mixed kernel (|dlnL| <= s |dX| at the window's
// samples): the float32 transform's rounding grows as ||z||_2 where the
// outputs are noise, and as the output itself at a peak of |X|, where every
// stage's terms add coherently (the window sums are compensated, so the
// column transforms' eleven stages dominate).  The coefficients hold with a
// margin of 2.3 or more over the measured errors of 8192 relative-binning
// draws (tf2_128s, time marginalisation; prior draws and loud templates
// between 5 and 120 Mpc with |X| up to 1.9e4).
constexpr double kWinErrNorm = 6e-7;
constexpr double kWinErrPeak = 2e-7;
// ... plus, for multi-banding, the independent relative errors (below about
// 2.5e-7) of the banded terms (phase fraction, sincospi, weight, products):
// four standard deviations of their sum over the window's samples
constexpr double kWinErrTerm = 1e-6;

namespace {

// A shared-memory layout of one CTA (byte offsets; every region 16-aligned).
struct WinLayout {
  int64_t n1;        // N1 columns
  int log2n2;        // column length N2 = 2^log2n2
  int n_win_max;     // accumulator slots (window samples)
  int n_otw_hi;      // mixed: entries of the coarse output twiddle table
  int off_ctw, off_otw_hi, off_otw_lo, off_acc, off_q, off_rat, off_coef, off_knots;
  int bytes;
};

// Columns per pass (the full-grid TaylorF2 source: one, its band being a few
// hundred bins of short transforms) and the column length's limit.
template <bool MIXED, int SRC>
__host__ __device__ constexpr int win_columns() {
  return SRC == 2 ? 1 : (MIXED ? 4 : 2);
}

template <bool MIXED, int SRC>
__host__ __device__ constexpr int win_max_log2_col() {
  return 11;
}

// radix-2 stages evaluated with the integrand, in registers
template <bool MIXED>
__host__ __device__ constexpr int win_first_stages() {
  return MIXED ? 4 : 3;
}

// padding: one slot after every 16 elements of a column; the columns are
// win_stride(N2) elements apart, 4 more than a multiple of 16, so that the G
// columns' blocks written by one half-warp fall in different banks

__device__ __forceinline__ int win_pad(int q) { return q + (q >> 4); }
__host__ __device__ constexpr int win_stride(int n2) { return n2 + n2 / 16 + 4; }

// s + e += y with s + e kept as an unevaluated float pair (Knuth's TwoSum;
// the adds are explicit so that nothing is contracted or reordered)
__device__ __forceinline__ void two_sum_acc(float& s, float& e, float y) {
  const float t = __fadd_rn(s, y);
  const float bp = __fsub_rn(t, s);
  const float err = __fadd_rn(__fsub_rn(s, __fsub_rn(t, bp)), __fsub_rn(y, bp));
  s = t;
  e = __fadd_rn(e, err);
}

template <class C>
__device__ __forceinline__ C cmul(C a, C b) {
  C r;
  r.x = a.x * b.x - a.y * b.y;
  r.y = a.x * b.y + a.y * b.x;
  return r;
}

// One in-place radix-2^RB pass (radix-2 stages stage .. stage + RB - 1,
// decimation in time) over the G columns of cs elements each.  ctw holds the
// stage tables: ctw[(h - 1) + p] = exp(-2 pi i p / (2 h)) for half-length h
// and p < h.
template <int RB, int G, class C>
__device__ __forceinline__ void win_pass(C* cols, int cs, int log2n2, int stage, const C* ctw) {
  constexpr int RN = 1 << RB;
  const int lpc = log2n2 - RB;  // log2 of the groups per column
  const int h0 = 1 << (stage - 1);
  for (int gi = threadIdx.x; gi < (G << lpc); gi += blockDim.x) {
    const int g = gi >> lpc, li = gi & ((1 << lpc) - 1);
    C* col = cols + g * cs;
    const int pos = li & (h0 - 1);
    const int b0 = ((li >> (stage - 1)) << (stage - 1 + RB)) + pos;
    C x[RN];
#pragma unroll
    for (int k = 0; k < RN; ++k) x[k] = col[win_pad(b0 + k * h0)];
#pragma unroll
    for (int j = 0; j < RB; ++j) {
      const int h = h0 << j;
#pragma unroll
      for (int k = 0; k < RN; ++k) {
        if (k & (1 << j)) continue;
        const int k2 = k | (1 << j);
        const C w = ctw[(h - 1) + pos + (k & ((1 << j) - 1)) * h0];
        const C t = cmul(w, x[k2]);
        x[k2].x = x[k].x - t.x;
        x[k2].y = x[k].y - t.y;
        x[k].x = x[k].x + t.x;
        x[k].y = x[k].y + t.y;
      }
    }
#pragma unroll
    for (int k = 0; k < RN; ++k) col[win_pad(b0 + k * h0)] = x[k];
  }
}

// The integrand's source: relative binning, multi-banding, or the TaylorF2
// model on the full frequency grid.
constexpr int kSrcRelbin = 0, kSrcMultiband = 1, kSrcTf2 = 2;

template <int D, bool MIXED, int SRC>
__global__ void __launch_bounds__(kWinThreads, MIXED ? 2 : 1)
    k_tm_window(LaunchArgs a, WinLayout lay, const typename TmTypes<MIXED>::C* twiddle) {
  using C = typename TmTypes<MIXED>::C;
  using R = typename TmTypes<MIXED>::R;
  constexpr int G = win_columns<MIXED, SRC>();
  constexpr int RB0 = win_first_stages<MIXED>(), RN0 = 1 << RB0;
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ C s_w16[16];
  __shared__ double s_red[2 * kWinWarps];
  __shared__ double s_scal[4];
  __shared__ long long s_jr[2];
  __shared__ long long s_kb[2];
  __shared__ int s_last;
  __shared__ SplineRowF s_row;
  __shared__ int s_tband[2];  // full-grid TaylorF2: the point's band
  const int L = (int)a.n_fft, N1 = (int)lay.n1;  // L < 2^30 (checked on the host)
  const int log2n2 = lay.log2n2;
  const int N2 = 1 << log2n2, n2q = N2 >> RB0, cs = win_stride(N2);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  C* cols = reinterpret_cast<C*>(smem);
  C* ctw = reinterpret_cast<C*>(smem + lay.off_ctw);
  C* acc = reinterpret_cast<C*>(smem + lay.off_acc);
  C* acc_lo = acc + lay.n_win_max;  // mixed: compensation of the window sums
  int* qst = reinterpret_cast<int*>(smem + lay.off_q);
  float2* otw_hi = reinterpret_cast<float2*>(smem + lay.off_otw_hi);
  float2* otw_lo = reinterpret_cast<float2*>(smem + lay.off_otw_lo);
  float* s_tx = reinterpret_cast<float*>(smem + lay.off_knots);
  float* s_ty = s_tx + a.nx;

  // Work units.  Evaluation: one per point.  Float64 recomputation of the
  // points the mixed kernel marked (rf_list[0 .. *rf_count)): P units per
  // point, unit c taking the column groups c, c + P, ...; each writes its
  // window sums and <h|h> share to tw_part, and the last of the point's units
  // to finish adds the P shares in a fixed order and completes the point.
  int P = 1;
  int64_t n_units = a.B;
  if (a.tw_refine_only) {
    const int64_t cnt = *a.rf_count;
    const int64_t groups = (N1 + G - 1) / G;
    // at least four column groups per unit (each unit repeats the per-point set-up)
    if (cnt > 0) P = (int)std::max<int64_t>(1, std::min<int64_t>(groups / 4, (int64_t)gridDim.x / cnt));
    if (cnt * P > a.tw_part_units) P = (int)std::max<int64_t>(1, a.tw_part_units / std::max<int64_t>(cnt, 1));
    n_units = cnt * P;
  }
  if ((int64_t)blockIdx.x >= n_units) return;  // no work for this CTA (uniform)

  // ---- tables, once per CTA ----------------------------------------------
  for (int e = threadIdx.x; e < N2 - 1; e += blockDim.x) {
    const int h = 1 << (31 - __clz(e + 1));  // largest power of two <= e + 1
    ctw[e] = twiddle[(e - (h - 1)) * (L / (2 * h))];
  }
  if (threadIdx.x < 8) {
    // exp(-2 pi i m / 16), m < 16
    const C t = twiddle[threadIdx.x * (L / 16)];
    s_w16[threadIdx.x] = t;
    C n;
    n.x = -t.x;
    n.y = -t.y;
    s_w16[threadIdx.x + 8] = n;
  }
  if constexpr (MIXED) {
    for (int q = threadIdx.x; q < lay.n_otw_hi; q += blockDim.x)
      otw_hi[q] = reinterpret_cast<const float2*>(twiddle)[q * kWinOutRows];
    for (int q = threadIdx.x; q < kWinOutRows; q += blockDim.x)
      otw_lo[q] = q < L / 2 ? reinterpret_cast<const float2*>(twiddle)[q] : make_float2(1.f, 0.f);
    if (a.dist_marg) {
      for (int q = threadIdx.x; q < a.nx; q += blockDim.x) s_tx[q] = a.tx_f[q];
      for (int q = threadIdx.x; q < a.ny; q += blockDim.x) s_ty[q] = a.ty_f[q];
    }
  }
  __syncthreads();
  // exp(-2 pi i q / L), 0 <= q < L
  const auto w_out = [&](int q) -> C {
    const bool neg = q >= L / 2;
    if (neg) q -= L / 2;
    C w;
    if constexpr (MIXED) {
      w = cmul(otw_hi[q / kWinOutRows], otw_lo[q % kWinOutRows]);
    } else {
      w = twiddle[q];
    }
    if (neg) {
      w.x = -w.x;
      w.y = -w.y;
    }
    return w;
  };

  const double norm = 4.0 / a.duration;
  const int nE = a.rb_edges, nB = nE - 1;
  constexpr bool MB = SRC == kSrcMultiband;
  const int k0 = SRC == kSrcRelbin ? (int)a.rb_index[0] : 0, k1 = SRC == kSrcRelbin ? (int)a.rb_index[nE - 1] : -1;
  for (int64_t unit = blockIdx.x; unit < n_units; unit += gridDim.x) {
    const int64_t slot = unit / P;
    const int part_c = (int)(unit - slot * P);
    const int64_t i = a.tw_refine_only ? (int64_t)a.rf_list[slot] : unit;
    const PointRec& r = a.rec[i];
    if (!r.valid) {
      if (threadIdx.x == 0 && part_c == 0) a.out[i] = -1.7976931348623157e308;  // nan_to_num(-inf)
      continue;
    }
    const double jit = r.jitter;
    if (threadIdx.x == 0) {
      // the candidate window of FFT indices (each sample is checked exactly below)
      const double step = a.duration / (double)L;
      const double jl = floor((a.t_min - a.start_time0 - jit) / step) - 3.0;
      const double jh = ceil((a.t_max - a.start_time0 - jit) / step) + 2.0;
      long long lo = (long long)fmax(0.0, jl), hi = (long long)fmin((double)(L - 1), jh);
      if (hi - lo + 1 > lay.n_win_max) {  // not reached: the host sizes the window from the prior
        atomicExch(a.status, kDevStatusBadInput);
        hi = lo + lay.n_win_max - 1;
      }
      s_jr[0] = lo;
      s_jr[1] = hi;
      s_scal[0] = step;
    }
    // ---- per-point set-up ----------------------------------------------
    // (multi-banding with the IFFT-FFT <h|h>: its odd-bin part, once)
    double hh_part = MB && part_c == 0 && threadIdx.x == 0 ? mb_fft_hh_total(a, i) : 0.0;
    float z2 = 0.f;  // mixed: sum of |z_k|^2 (error bound)
    double2* rat = reinterpret_cast<double2*>(smem + lay.off_rat);  // relative binning: [D][nE]
    float4* coef = reinterpret_cast<float4*>(smem + lay.off_coef);  // mixed: [D][nB] {r0, r1}, then [D][nB] lo(r0)
    if constexpr (SRC == kSrcRelbin) {
      relbin_edge_ratios<D>(a, r, rat);
      __syncthreads();
      if (part_c == 0) hh_part = relbin_hh_part<D>(a, rat);
      if constexpr (MIXED) {
        // relative.py:374-377: r0 = (q_b+1 + q_b) / 2, r1 = (q_b+1 - q_b) / width;
        // r0 as float-float (its rounding would be the same for every grid
        // index of the bin and add up coherently), r1 (f - f_b) is small
        float2* coef_lo = reinterpret_cast<float2*>(coef + D * nB);
        for (int t = threadIdx.x; t < D * nB; t += blockDim.x) {
          const int d = t / nB, b = t - d * nB;
          const double2 q0 = rat[d * nE + b], q1 = rat[d * nE + b + 1];
          const double width = a.rb_freq[b + 1] - a.rb_freq[b];
          const double r0r = (q1.x + q0.x) / 2, r0i = (q1.y + q0.y) / 2;
          const float hr = (float)r0r, hi = (float)r0i;
          coef[t] = make_float4(hr, hi, (float)((q1.x - q0.x) / width), (float)((q1.y - q0.y) / width));
          coef_lo[t] = make_float2((float)(r0r - (double)hr), (float)(r0i - (double)hi));
        }
      }
    }
    // mixed multi-banding: z_m = sum_d A Q_d exp(-i phase_d(f_m)) L_d(f_m) at
    // every banded frequency m into this CTA's slot of the work space
    // (L2-resident), as k_multiband_mixed forms its terms: the TaylorF2 phase
    // from the float-float basis, detector d's time shift exact in 0.64 fixed
    // point per band, sincospi of the exact fraction; <h|h> from the prefix
    // sums of the quadratic coefficients over the point's band.
    float2* zb = nullptr;
    if constexpr (MIXED && MB) {
      {
        zb = a.tw_scratch + (size_t)blockIdx.x * (size_t)a.mb_points;
        uint64_t* s_y = reinterpret_cast<uint64_t*>(smem + lay.off_rat);  // [bands][D]: frac(f_b0 dt_d)
        uint64_t* s_x = s_y + a.mb_bands * D;                              // [bands][D]: frac(df_b dt_d)
        float2* s_g = reinterpret_cast<float2*>(s_x + a.mb_bands * D);     // [D]: A Q_d scale_d
        for (int t = threadIdx.x; t < a.mb_bands * D; t += blockDim.x) {
          const int b = t / D, d = t - b * D;
          const double y = a.mb_freq[a.mb_band_start[b]] * r.dt[d], x = a.mb_band_df[b] * r.dt[d];
          double fy = ldexp(y - floor(y), 64), fx = ldexp(x - floor(x), 64);
          if (!(fy < 18446744073709551616.0)) fy = 0.0;
          if (!(fx < 18446744073709551616.0)) fx = 0.0;
          s_y[t] = (uint64_t)fy;
          s_x[t] = (uint64_t)fx;
        }
        if (threadIdx.x == 32) {
          // the point's band among the banded frequencies: fmin <= f < f_isco
          int64_t lo = 0, hi = a.mb_points;
          while (lo < hi) {
            const int64_t mid = (lo + hi) / 2;
            if (a.mb_freq[mid] >= a.fmin) hi = mid; else lo = mid + 1;
          }
          const int64_t kb0 = lo;
          hi = a.mb_points;
          while (lo < hi) {
            const int64_t mid = (lo + hi) / 2;
            if (a.mb_freq[mid] >= r.f_isco) hi = mid; else lo = mid + 1;
          }
          const int64_t kb1 = lo;
          s_kb[0] = kb0;
          s_kb[1] = kb1;
          const double ci = r.cos_i, pfac = (1.0 + ci * ci) / 2.0;
          for (int d = 0; d < D; ++d) {
            const double qr = r.fp[d] * pfac, qi = -r.fx[d] * ci;
            s_g[d] = make_float2((float)(r.amp * qr * a.mb_lw_scale[d]), (float)(r.amp * qi * a.mb_lw_scale[d]));
            hh_part += r.amp * r.amp * (qr * qr + qi * qi) * (a.mb_qprefix[d][kb1] - a.mb_qprefix[d][kb0]);
          }
        }
        float ch[kNumBasis + 1], cl[kNumBasis + 1];
#pragma unroll
        for (int b = 0; b <= kNumBasis; ++b) {
          ch[b] = r.c_hi[b];
          cl[b] = r.c_lo[b];
        }
        __syncthreads();
        const int64_t kb0 = s_kb[0], kb1 = s_kb[1];
        for (int b = 0; b < a.mb_bands; ++b) {
          const int64_t bs = a.mb_band_start[b], be = a.mb_band_start[b + 1];
          for (int64_t m = bs + threadIdx.x; m < be; m += blockDim.x) {
            float2 z = make_float2(0.f, 0.f);
            if (m >= kb0 && m < kb1) {
              const float4* bp = reinterpret_cast<const float4*>(a.mb_basis + m * kNumBasis);
              float s_hi = ch[kNumBasis], s_lo = cl[kNumBasis];
#pragma unroll
              for (int q = 0; q < kNumBasis / 2; ++q) {
                const float4 v = __ldg(bp + q);
                ff_mac(s_hi, s_lo, ch[2 * q], cl[2 * q], v.x, v.y);
                ff_mac(s_hi, s_lo, ch[2 * q + 1], cl[2 * q + 1], v.z, v.w);
              }
              const uint64_t base = to_fixed(s_hi, s_lo), idx = (uint64_t)(m - bs);
#pragma unroll
              for (int d = 0; d < D; ++d) {
                const uint64_t full = base + s_y[b * D + d] + idx * s_x[b * D + d];
                const uint32_t top = (uint32_t)((full + 0x80000000ull) >> 32);
                const float ph = __fmul_rn(__int2float_rn((int)top), 4.656612873077393e-10f);  // 2 * 2^-32
                float sn, cs;
                sincospif(ph, &sn, &cs);
                const float2 Lw = __ldg(a.mb_lw[d] + m);
                // exp(-i 2 pi frac) L, then times A Q_d scale_d
                const float tr = cs * Lw.x + sn * Lw.y, ti = cs * Lw.y - sn * Lw.x;
                const float2 g = s_g[d];
                z.x += g.x * tr - g.y * ti;
                z.y += g.x * ti + g.y * tr;
              }
              z2 += z.x * z.x + z.y * z.y;
            }
            zb[m] = z;
          }
        }
        __syncthreads();
      }
    }
    if constexpr (SRC == kSrcTf2) {
      if (threadIdx.x == 32) {
        s_tband[0] = (int)max(r.k_start, a.k_lo);
        s_tband[1] = (int)min(min(r.k_end, a.k_hi), (int64_t)L);
        if (!MIXED && part_c == 0 && L >= a.k_lo && L < a.k_hi) {
          // the last bin (index L) enters <h|h> only; the transform uses bins 0 .. L - 1
          double2 hp, hx;
          const double f = a.freq[L];
          if (plain_pols(a, r, f, hp, hx)) {
            for (int d = 0; d < D; ++d) {
              const double sre = hp.x * r.fp[d] + hx.x * r.fx[d], sim = hp.y * r.fp[d] + hx.y * r.fx[d];
              hh_part += norm * (sre * sre + sim * sim) * a.inv_psd[d][L];
            }
          }
        }
      }
      __syncthreads();
    }
    const bool tf2 = a.model == GWL_MODEL_TAYLORF2;
    const bool pw = SRC != kSrcRelbin && !MIXED && tf2;  // float64 model from the power tables
    const double u = pw ? cbrt(kPi * r.m_sec) : 0.0;
    const double lnu = pw ? log(u) : 0.0;
    const double pu5 = pw ? 3.0 / (128.0 * r.eta) / (u * u * u * u * u) : 0.0;
    for (int t = threadIdx.x; t < lay.n_win_max; t += blockDim.x) {
      C z;
      z.x = 0;
      z.y = 0;
      acc[t] = z;
      if constexpr (MIXED) acc_lo[t] = z;
      qst[t] = 0;
    }
    __syncthreads();
    const int j_lo = (int)s_jr[0];
    const int n_win = (int)(s_jr[1] - s_jr[0] + 1);
    // integrand z_k (k < L): 4/T sum_d h_d,k conj(d_k) / S_k
    const auto integrand = [&](int k) -> C {
      C z;
      z.x = 0;
      z.y = 0;
      if constexpr (SRC == kSrcTf2) {
        if (k < s_tband[0] || k >= s_tband[1]) return z;
        if constexpr (!MIXED) {
          // float64 (base.py:325-330): the model from the per-bin power
          // table, the detector response with its time shift, h conj(d) / S
          // (the recomputation of the points the mixed whole-FFT kernel marks)
          const double f = a.freq[k];
          double2 hp, hx;
          if (tf2_pols_tab(a, r, k, f, u, lnu, pu5, hp, hx)) {
            double zr = 0.0, zi = 0.0, hs = 0.0;
#pragma unroll
            for (int d = 0; d < D; ++d) {
              const double is = a.inv_psd[d][k];
              if (is == 0.0) continue;
              const double sre = hp.x * r.fp[d] + hx.x * r.fx[d], sim = hp.y * r.fp[d] + hx.y * r.fx[d];
              double sn, cs;
              sincos(2.0 * kPi * r.dt[d] * f, &sn, &cs);
              const double hre = sre * cs + sim * sn, him = sim * cs - sre * sn;
              const double2 dd = reinterpret_cast<const double2*>(a.strain[d])[k];
              zr += (hre * dd.x + him * dd.y) * is;
              zi += (him * dd.x - hre * dd.y) * is;
              hs += (hre * hre + him * him) * is;
            }
            z.x = norm * zr;
            z.y = norm * zi;
            hh_part += norm * hs;
          }
        }
        return z;
      } else if constexpr (!MB) {
        if constexpr (MIXED) {
          // float32: ratio r0 + r1 (f - f_b) times the weight 4/T h0 conj(d) / S;
          // no branch around the loads (a clamped index and a zero factor
          // outside the bins' span), so that those of several k are in flight
          const int kc = min(max(k, k0), k1) - k0;
          const float in = (k >= k0 && k <= k1) ? 1.f : 0.f;
          const float2 bxw = __ldg(reinterpret_cast<const float2*>(a.rb_bx) + kc);
          const RbBinF bx{__float_as_int(bxw.x), bxw.y};
          const float2* coef_lo = reinterpret_cast<const float2*>(coef + D * nB);
#pragma unroll
          for (int d = 0; d < D; ++d) {
            const float4 c = coef[d * nB + bx.bin];
            const float2 cl = coef_lo[d * nB + bx.bin];
            const float rr = fmaf(c.z, bx.x, c.x) + cl.x, ri = fmaf(c.w, bx.x, c.y) + cl.y;
            const float2 g = __ldg(a.rb_gf[d] + kc);
            z.x += g.x * rr - g.y * ri;
            z.y += g.x * ri + g.y * rr;
          }
          z.x *= in;
          z.y *= in;
          z2 += z.x * z.x + z.y * z.y;
        } else {
          if (k < k0 || k > k1) return z;
          // relative.py:380-396: h0_d(f) (r0_b + r1_b (f - f_b)) of bin b
          const int b = a.rb_bin[k - k0];
          if (!GWL_INDEX_OK(b, nE - 1, a.status)) return z;
          const double fb0 = a.rb_freq[b], fb1 = a.rb_freq[b + 1];
          const double x = a.freq[k] - (fb1 + fb0) / 2, width = fb1 - fb0;
#pragma unroll
          for (int d = 0; d < D; ++d) {
            const double2 q0 = rat[d * nE + b], q1 = rat[d * nE + b + 1];
            const double rr = (q1.x + q0.x) / 2 + (q1.x - q0.x) / width * x;
            const double ri = (q1.y + q0.y) / 2 + (q1.y - q0.y) / width * x;
            const double2 g = a.rb_g[d][k];  // 4/T h0 conj(d) / S
            z.x += g.x * rr - g.y * ri;
            z.y += g.x * ri + g.y * rr;
          }
        }
        return z;
      }
      if constexpr (MIXED) {
        // multi-banding: the banded values at the full-resolution indices
        // int(f_m T) (multiband.py:714-726)
        const int32_t c1 = a.mb_tm_ptr[k + 1];
        for (int32_t c = a.mb_tm_ptr[k]; c < c1; ++c) {
          const int32_t code = a.mb_tm_src[c];
          if (code >= 0 && GWL_INDEX_OK(code, a.mb_points, a.status)) {
            const float2 v = zb[code];
            z.x += v.x;
            z.y += v.y;
          }
        }
      } else {
        // multi-banding: the banded strain times the linear coefficients at the
        // full-resolution indices int(f_j T); <h|h> from the quadratic ones
        const int32_t c1 = a.mb_tm_ptr[k + 1];
        for (int32_t c = a.mb_tm_ptr[k]; c < c1; ++c) {
          const int32_t code = a.mb_tm_src[c];
          const int64_t jb = code >= 0 ? (int64_t)code : -(int64_t)code - 1;
          if (!GWL_INDEX_OK(jb, a.mb_points, a.status)) continue;
          const double f = a.mb_freq[jb];
          double2 hp = make_double2(0.0, 0.0), hx = make_double2(0.0, 0.0);
          if (!(tf2 ? tf2_pols_t(a, r, a.mb_pow[jb], f, u, lnu, pu5, hp, hx) : plain_pols(a, r, f, hp, hx))) continue;
#pragma unroll
          for (int d = 0; d < D; ++d) {
            // interferometer.py:341-362 at explicit frequencies (no mask)
            const double sre = hp.x * r.fp[d] + hx.x * r.fx[d], sim = hp.y * r.fp[d] + hx.y * r.fx[d];
            double sn, cs;
            sincos(2.0 * kPi * r.dt[d] * f, &sn, &cs);
            const double hre = sre * cs + sim * sn, him = sim * cs - sre * sn;
            hh_part += (hre * hre + him * him) * a.mb_quad[d][jb];
            if (code >= 0) {
              const double2 w = a.mb_lin[d][jb];
              z.x += hre * w.x - him * w.y;
              z.y += hre * w.y + him * w.x;
            }
          }
        }
      }
      return z;
    };

    // ---- columns: integrand, transform, window sums ------------------------
    for (int n1_0 = part_c * G; n1_0 < N1; n1_0 += P * G) {
      // A block b of RN0 positions of column g holds, after the first RB0
      // stages, the RN0-point DFT of the column's elements q + m N2 / RN0
      // (m < RN0), q = bitrev(b) over log2(N2) - RB0 bits.
      for (int bb = threadIdx.x; bb < G * n2q; bb += blockDim.x) {
        const int g = bb % G, b = bb / G, n1 = n1_0 + g;
        const int q = log2n2 > RB0 ? (int)bit_reverse((uint32_t)b, log2n2 - RB0) : 0;
        C x[RN0];
        if constexpr (SRC == kSrcTf2) {
          // the band is a few hundred of the column's bins: a block with none
          // of its RN0 elements (N1 N2 / RN0 apart) in it writes zeros
          const int64_t kmin = (int64_t)n1 + (int64_t)N1 * q, stride = (int64_t)N1 * n2q;
          const int64_t lo = (int64_t)s_tband[0] - kmin, hi = (int64_t)s_tband[1] - kmin;
          const int64_t m_lo = lo <= 0 ? 0 : (lo + stride - 1) / stride, m_hi = hi <= 0 ? -1 : (hi - 1) / stride;
          if (n1 >= N1 || m_lo > min(m_hi, (int64_t)RN0 - 1)) {
            C* col = cols + g * cs;
            C zero;
            zero.x = 0;
            zero.y = 0;
#pragma unroll
            for (int m = 0; m < RN0; ++m) col[win_pad(b * RN0 + m)] = zero;
            continue;
          }
        }
#pragma unroll
        for (int m = 0; m < RN0; ++m) {
          // register slot m holds element bitrev(m) (decimation in time)
          const int mm = (int)(__brev((unsigned)m) >> (32 - RB0));
          if (n1 < N1) {
            x[m] = integrand(n1 + N1 * (q + mm * n2q));
          } else {
            x[m].x = 0;
            x[m].y = 0;
          }
        }
#pragma unroll
        for (int s = 0; s < RB0; ++s) {
          const int h = 1 << s;
#pragma unroll
          for (int k = 0; k < RN0; ++k) {
            if (k & h) continue;
            // exp(-2 pi i (k mod h) / (2 h)) = w16[(k mod h) 16 / (2 h)]
            const C w = s_w16[(k & (h - 1)) * (8 >> s)];
            const C t = cmul(w, x[k | h]);
            x[k | h].x = x[k].x - t.x;
            x[k | h].y = x[k].y - t.y;
            x[k].x = x[k].x + t.x;
            x[k].y = x[k].y + t.y;
          }
        }
        C* col = cols + g * cs;
#pragma unroll
        for (int m = 0; m < RN0; ++m) col[win_pad(b * RN0 + m)] = x[m];
      }
      __syncthreads();
      for (int stage = RB0 + 1; stage <= log2n2;) {
        const int rem = log2n2 - stage + 1;
        if (MIXED && rem >= 4) {
          win_pass<4, G>(cols, cs, log2n2, stage, ctw);
          stage += 4;
        } else if (rem >= 3) {
          win_pass<3, G>(cols, cs, log2n2, stage, ctw);
          stage += 3;
        } else if (rem == 2) {
          win_pass<2, G>(cols, cs, log2n2, stage, ctw);
          stage += 2;
        } else {
          win_pass<1, G>(cols, cs, log2n2, stage, ctw);
          stage += 1;
        }
        __syncthreads();
      }
      // X[j] += sum_g exp(-2 pi i n1 j / L) B_n1[j mod N2]; qst[t] = n1 j mod L.
      // Mixed: compensated sums (the N1 terms add up coherently at a peak of
      // |X|, where plain float32 sums would lose sqrt(N1) ulps), the
      // compensation in acc_lo.
      for (int t = threadIdx.x; t < n_win; t += blockDim.x) {
        const int j = j_lo + t, jm = j & (N2 - 1);
        // n1 j mod L: carried from the previous group, or (a unit of a split
        // recomputation, whose groups are P apart) formed afresh
        int qq = P > 1 ? (int)(((int64_t)n1_0 * j) % L) : qst[t];
        C s = acc[t], e;
        if constexpr (MIXED) e = acc_lo[t];
#pragma unroll
        for (int g = 0; g < G; ++g) {
          if (n1_0 + g < N1) {
            const C y = cmul(w_out(qq), cols[g * cs + win_pad(jm)]);
            if constexpr (MIXED) {
              two_sum_acc(s.x, e.x, y.x);
              two_sum_acc(s.y, e.y, y.y);
            } else {
              s.x += y.x;
              s.y += y.y;
            }
            qq += j;
            if (qq >= L) qq -= L;
          }
        }
        acc[t] = s;
        if constexpr (MIXED) acc_lo[t] = e;
        qst[t] = qq;
      }
      __syncthreads();
    }

    // ---- <h|h>, error norm, per-sample lnL, logsumexp ------------------------
    double hh = hh_part;
    float zz = z2;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      hh += __shfl_xor_sync(0xffffffffu, hh, o);
      zz += __shfl_xor_sync(0xffffffffu, zz, o);
    }
    if (lane == 0) {
      s_red[warp] = hh;
      s_red[kWinWarps + warp] = (double)zz;
    }
    __syncthreads();
    if (threadIdx.x == 0 || threadIdx.x == 32) {
      double h = 0.0, n2 = 0.0;
      for (int w = 0; w < kWinWarps; ++w) {
        h += s_red[w];
        n2 += s_red[kWinWarps + w];
      }
      const double sr = r.dist / a.ref_dist;
      if (threadIdx.x == 0) {
        s_scal[1] = h;
        s_scal[2] = sr;
        s_scal[3] = sqrt(n2);
      } else if (MIXED && a.dist_marg) {
        s_row = bicubic_row_f(s_ty, a.ny, a.bbox, (float)(h * sr * sr));
      }
    }
    __syncthreads();
    if (P > 1) {
      // this unit's share to the point's slot; the last unit adds them up
      double2* share = reinterpret_cast<double2*>(a.tw_part) + (size_t)unit * (lay.n_win_max + 1);
      for (int t = threadIdx.x; t < n_win; t += blockDim.x) share[t] = make_double2(acc[t].x, acc[t].y);
      if (threadIdx.x == 0) share[lay.n_win_max] = make_double2(s_scal[1], 0.0);
      __threadfence();
      __syncthreads();
      if (threadIdx.x == 0) s_last = atomicAdd(a.tw_done + slot, 1) == P - 1;
      __syncthreads();
      if (!s_last) continue;  // uniform over the CTA
      __threadfence();
      const double2* shares = reinterpret_cast<const double2*>(a.tw_part) + (size_t)slot * P * (lay.n_win_max + 1);
      for (int t = threadIdx.x; t < n_win; t += blockDim.x) {
        double xr = 0.0, xi = 0.0;
        for (int c = 0; c < P; ++c) {
          const double2 v = __ldcg(shares + (size_t)c * (lay.n_win_max + 1) + t);
          xr += v.x;
          xi += v.y;
        }
        acc[t].x = (R)xr;
        acc[t].y = (R)xi;
      }
      if (threadIdx.x == 0) {
        double h = 0.0;
        for (int c = 0; c < P; ++c) h += __ldcg(shares + (size_t)c * (lay.n_win_max + 1) + lay.n_win_max).x;
        s_scal[1] = h;
      }
      __syncthreads();
    }
    const double step = s_scal[0], hh_all = s_scal[1], sr = s_scal[2], znorm = s_scal[3];
    const double hh_ref = hh_all * sr * sr;
    double m = -INFINITY, lse = 0.0;
    float xmax = 0.f;
    for (int t = threadIdx.x; t < n_win; t += blockDim.x) {
      const int j = j_lo + t;
      const double tj = tm_sample_time(a, j, L, step, jit);
      double lw;
      if (!tm_log_weight<MIXED>(a, tj, lw)) continue;
      C x = acc[t];
      if constexpr (MIXED) {
        x.x += acc_lo[t].x;
        x.y += acc_lo[t].y;
      }
      double l;
      if constexpr (MIXED) {
        l = tm_lnl_mixed(a, x.x, x.y, hh_all, sr, s_tx, s_row);
        xmax = fmaxf(xmax, sqrtf(x.x * x.x + x.y * x.y));
      } else {
        l = tm_lnl_fp64(a, x.x, x.y, hh_all, hh_ref, sr);
      }
      tm_lse_push<MIXED>(l + lw, m, lse);
    }
    // the block's maximum M, then sum_t lse_t exp(m_t - M) in a fixed order
    double mx = m;
    float xm = xmax;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
      xm = fmaxf(xm, __shfl_xor_sync(0xffffffffu, xm, o));
    }
    __syncthreads();
    if (lane == 0) {
      s_red[warp] = mx;
      s_red[kWinWarps + warp] = (double)xm;
    }
    __syncthreads();
    double M = s_red[0];
    for (int w = 1; w < kWinWarps; ++w) M = fmax(M, s_red[w]);
    double xpk = 0.0;
    if (threadIdx.x == 0)
      for (int w = 0; w < kWinWarps; ++w) xpk = fmax(xpk, s_red[kWinWarps + w]);
    double sm = 0.0;
    if (isfinite(M) && isfinite(m)) sm = lse * (MIXED ? (double)__expf((float)(m - M)) : exp(m - M));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) sm += __shfl_xor_sync(0xffffffffu, sm, o);
    __syncthreads();
    if (lane == 0) s_red[warp] = sm;
    __syncthreads();
    if (threadIdx.x == 0) {
      double total = 0.0;
      for (int w = 0; w < kWinWarps; ++w) total += s_red[w];
      total *= (a.tm_prior ? 1.0 : 1.0 / (a.t_max - a.t_min)) * a.delta_tc;
      double lnl;
      if (!isfinite(M)) lnl = M;
      else lnl = M + log(total);
      a.out[i] = lnl;
      if (MIXED && a.rf_tol > 0 && a.rf_count) {
        // |dlnL| <= max_j |dl_j| <= s |dX|max
        const double sens = tm_sensitivity(a, xpk, sr, s_tx, s_row);
        const double err = (kWinErrNorm + (SRC != kSrcRelbin ? kWinErrTerm : 0.0)) * znorm + kWinErrPeak * xpk;
        if (!(sens * err <= a.rf_tol)) {
          a.rec[i].refine = 1;
          a.rf_list[atomicAdd(a.rf_count, 1)] = (int32_t)i;
        }
      }
    }
    __syncthreads();
  }
}

// Shared-memory layout for n_det detectors; false when it does not fit.
template <bool MIXED, int SRC>
bool win_layout(const LaunchArgs& a, WinLayout* lay) {
  using C = typename TmTypes<MIXED>::C;
  int m_odd = 0, log2N = 0;
  if (!fft_length_supported(a.n_fft, &m_odd, &log2N) || a.n_fft >= ((int64_t)1 << 30)) return false;
  const int log2n2 = std::min(log2N, win_max_log2_col<MIXED, SRC>());
  const int64_t n2 = (int64_t)1 << log2n2;
  lay->log2n2 = log2n2;
  lay->n1 = a.n_fft >> log2n2;
  const double step = a.duration / (double)a.n_fft;
  const double width = (a.t_max - a.t_min) / step;
  if (!(width >= 0.0) || width > 1e6) return false;
  lay->n_win_max = (int)std::ceil(width) + 10;
  lay->n_otw_hi = (int)((a.n_fft / 2 + kWinOutRows - 1) / kWinOutRows);
  const auto up16 = [](size_t x) { return (x + 15) & ~(size_t)15; };
  size_t off = up16((size_t)win_columns<MIXED, SRC>() * (size_t)win_stride((int)n2) * sizeof(C));
  lay->off_ctw = (int)off;
  off = up16(off + (size_t)(n2 - 1) * sizeof(C));
  lay->off_otw_hi = (int)off;
  off = up16(off + (MIXED ? (size_t)lay->n_otw_hi * sizeof(float2) : 0));
  lay->off_otw_lo = (int)off;
  off = up16(off + (MIXED ? (size_t)kWinOutRows * sizeof(float2) : 0));
  lay->off_acc = (int)off;
  off = up16(off + (size_t)lay->n_win_max * sizeof(C) * (MIXED ? 2 : 1));
  lay->off_q = (int)off;
  off = up16(off + (size_t)lay->n_win_max * sizeof(int));
  lay->off_rat = (int)off;
  size_t rat = a.relbin ? (size_t)a.n_det * a.rb_edges * sizeof(double2) : 0;
  if (MIXED && a.mb_tm) rat = (size_t)a.mb_bands * a.n_det * 2 * sizeof(uint64_t) + (size_t)a.n_det * sizeof(float2);
  off = up16(off + rat);
  lay->off_coef = (int)off;
  off = up16(off + ((MIXED && a.relbin) ? (size_t)a.n_det * (a.rb_edges - 1) * (sizeof(float4) + sizeof(float2)) : 0));
  lay->off_knots = (int)off;
  off = up16(off + ((MIXED && a.dist_marg) ? (size_t)(a.nx + a.ny) * sizeof(float) : 0));
  lay->bytes = (int)off;
  return off <= (size_t)200 * 1024;
}

template <int D, bool MIXED, int SRC>
cudaError_t launch_win_d(const LaunchArgs& a, const WinLayout& lay, const TwiddleTables& tw, cudaStream_t s) {
  cudaError_t e =
      cudaFuncSetAttribute(k_tm_window<D, MIXED, SRC>, cudaFuncAttributeMaxDynamicSharedMemorySize, lay.bytes);
  if (e != cudaSuccess) return e;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  // the recomputation's unit count is known on the device only
  int64_t grid = a.tw_refine_only ? 8 * (int64_t)std::max(sms, 1) : std::min<int64_t>(a.B, 8 * (int64_t)std::max(sms, 1));
  if (MIXED && a.mb_tm) grid = std::min<int64_t>(grid, a.tw_scratch_slots);  // one work-space slot per CTA
  const typename TmTypes<MIXED>::C* twp;
  if constexpr (MIXED) twp = tw.d32;
  else twp = tw.d64;
  k_tm_window<D, MIXED, SRC><<<(unsigned)grid, kWinThreads, lay.bytes, s>>>(a, lay, twp);
  return cudaGetLastError();
}

template <bool MIXED, int SRC>
cudaError_t launch_win_src(const LaunchArgs& a, const WinLayout& lay, const TwiddleTables& tw, cudaStream_t s) {
  switch (a.n_det) {
    case 1: return launch_win_d<1, MIXED, SRC>(a, lay, tw, s);
    case 2: return launch_win_d<2, MIXED, SRC>(a, lay, tw, s);
    case 3: return launch_win_d<3, MIXED, SRC>(a, lay, tw, s);
    default: return launch_win_d<4, MIXED, SRC>(a, lay, tw, s);
  }
}

template <bool MIXED, int SRC>
cudaError_t launch_win_layout(const LaunchArgs& a, cudaStream_t s) {
  WinLayout lay;
  if (!win_layout<MIXED, SRC>(a, &lay)) return cudaErrorInvalidValue;  // checked on the host first
  TwiddleTables tw;
  cudaError_t e = twiddles_for(a.n_fft, &tw);
  if (e != cudaSuccess) return e;
  return launch_win_src<MIXED, SRC>(a, lay, tw, s);
}

int win_source(const LaunchArgs& a) { return a.relbin ? kSrcRelbin : (a.mb_tm ? kSrcMultiband : kSrcTf2); }

template <bool MIXED>
bool win_layout_any(const LaunchArgs& a, WinLayout* lay) {
  switch (win_source(a)) {
    case kSrcRelbin: return win_layout<MIXED, kSrcRelbin>(a, lay);
    case kSrcMultiband: return win_layout<MIXED, kSrcMultiband>(a, lay);
    default: return !MIXED && win_layout<false, kSrcTf2>(a, lay);
  }
}

template <bool MIXED>
cudaError_t launch_win(const LaunchArgs& a, cudaStream_t s) {
  switch (win_source(a)) {
    case kSrcRelbin: return launch_win_layout<MIXED, kSrcRelbin>(a, s);
    case kSrcMultiband: return launch_win_layout<MIXED, kSrcMultiband>(a, s);
    default:
      if constexpr (MIXED) return cudaErrorInvalidValue;  // float64 only
      else return launch_win_layout<false, kSrcTf2>(a, s);
  }
}

}  // namespace

bool time_marg_window_mixed_ready(const LaunchArgs& a) {
  if (a.relbin) return a.rb_bx != nullptr;
  return a.mb_tm && a.model == GWL_MODEL_TAYLORF2 && a.mb_basis && a.tw_scratch && a.tw_scratch_slots > 0;
}

int64_t time_marg_window_slots() {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return 2 * (int64_t)std::max(sms, 1);  // the mixed kernel's resident CTAs
}

size_t time_marg_window_share_bytes(const LaunchArgs& a) {
  LaunchArgs F = a;
  F.precision = GWL_PRECISION_FP64;
  WinLayout lay;
  if (!win_layout_any<false>(F, &lay)) return 0;
  return (size_t)(lay.n_win_max + 1) * sizeof(double2);
}

bool time_marg_window_refine_fits(const LaunchArgs& a) {
  if (a.tm_series || a.roq) return false;
  LaunchArgs F = a;
  F.precision = GWL_PRECISION_FP64;
  WinLayout lay;
  return win_layout_any<false>(F, &lay);
}

bool time_marg_window_fits(const LaunchArgs& a) {
  // relative binning and multi-banding, either precision (the full-grid
  // TaylorF2 source serves only the recomputation of marked points)
  if (!(a.relbin || a.mb_tm) || a.tm_series) return false;
  WinLayout lay;
  return a.precision == GWL_PRECISION_MIXED ? win_layout_any<true>(a, &lay) : win_layout_any<false>(a, &lay);
}

cudaError_t launch_time_marg_window(const LaunchArgs& a, cudaStream_t s) {
  if (a.precision == GWL_PRECISION_MIXED) {
    if (!time_marg_window_mixed_ready(a)) return cudaErrorInvalidValue;  // checked on the host first
    return launch_win<true>(a, s);
  }
  return launch_win<false>(a, s);
}

}  // namespace gwl
