// Host runtime behind include/gwlnl.h: builds the device-resident tables of an
// analysis, owns its work space and sequences the kernels of one evaluation.
#include <cublas_v2.h>
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "gwl_internal.h"
#include "gwl_math.cuh"

namespace gwl {

static thread_local std::string t_last_error;

void set_error(const std::string& msg) { t_last_error = msg; }

#define GWL_CUDA(expr)                                                                   \
  do {                                                                                   \
    cudaError_t _e = (expr);                                                             \
    if (_e != cudaSuccess) {                                                             \
      set_error(std::string(#expr) + ": " + cudaGetErrorString(_e));                     \
      return GWL_ERR_CUDA;                                                               \
    }                                                                                    \
  } while (0)

// Compensated (Kahan-Babuska) float64 accumulator for the set-up sums.
struct KahanSum {
  double s = 0.0, c = 0.0;
  void add(double x) {
    const double t = s + x;
    if (std::fabs(s) >= std::fabs(x)) c += (s - t) + x; else c += (x - t) + s;
    s = t;
  }
  double value() const { return s + c; }
};

}  // namespace gwl

using namespace gwl;

struct gwl_analysis {
  int model = 0, n_det = 0;
  int64_t n_bins = 0, n_pad = 0, k_lo = 0, k_hi = 0, k_base = 0, k_fmin = 0;
  int64_t n_chunks_plain = 0, n_chunks_mixed = 0;
  double duration = 0, fs = 0, fmin = 0, step = 0, start0 = 0;
  DetGeom geom[kMaxDet];
  std::vector<std::vector<double>> host_strain;  // kept for the noise log-likelihood
  double noise_lnl = 0.0;
  // device tables
  double* freq = nullptr;
  float* freq_f = nullptr;
  float2* basis = nullptr;
  double4* ftab = nullptr;  // float64 TaylorF2: {f^(1/3), ln(f) / 3, f^(-5/3), f^(-7/6)} per bin
  float* anchors = nullptr;
  int64_t n_anchors = 0;
  double* strain[kMaxDet] = {};
  double* inv_psd[kMaxDet] = {};
  float2* w[kMaxDet] = {};
  uint2* wp[kMaxDet] = {};  // TaylorF2: the same weights in polar form {float |w|, arg(w) as 0.32 fixed cycles}
  uint4* wq[kMaxDet] = {};  // TaylorF2 fast kernel: bin pairs {|w|, |w|, angle or angle increment} (LaunchArgs::wq)
  float* v[kMaxDet] = {};
  float* v_lo[kMaxDet] = {};  // sine-Gaussian: low words of the scaled inverse PSD
  double* hh_prefix[kMaxDet] = {};
  double* rf_p2[kMaxDet] = {};  // TaylorF2: prefix sums of |w|^2 and of |w| over signal-dominated bins
  double* rf_p1[kMaxDet] = {};
  double refine_tol = kRefineDefaultTol;  // mixed-precision refinement tolerance (<= 0: off)
  float4* cos_tab = nullptr;  // TaylorF2: float-float cos / sin of 2 pi q / kCosTable (accurate kernel)
  double w_scale[kMaxDet] = {}, v_scale[kMaxDet] = {};
  // marginalisation
  int time_marg = 0, jitter = 0, phase_marg = 0, dist_marg = 0;
  double dist_slope = 1.0;  // d_ref / d_min of the distance prior (gwl_set_distance_slope)
  double t_min = 0, t_max = 0;
  double* tm_prior = nullptr;  // time prior density on a uniform grid (nullptr: Uniform)
  float* tm_prior_f = nullptr;
  int64_t tm_prior_n = 0;
  double tm_prior_t0 = 0, tm_prior_inv_h = 0;
  double* tx = nullptr;
  double* ty = nullptr;
  double* tc = nullptr;
  float* tx_f = nullptr;
  float* ty_f = nullptr;
  float* tc_f = nullptr;
  int nx = 0, ny = 0;
  double bbox[4] = {0, 0, 0, 0};
  double ref_dist = 0;
  // relative binning
  int relbin = 0;
  int rb_edges = 0;
  int64_t* rb_index = nullptr;
  double* rb_freq = nullptr;
  double2* rb_h0inv[kMaxDet] = {};
  double* rb_sum[kMaxDet] = {};
  std::vector<int64_t> h_rb_index;  // host copy of the edges
  int rb_tm = 0;                    // time-marginalisation weights set for these bins
  double2* rb_g[kMaxDet] = {};
  int32_t* rb_bin = nullptr;
  float2* rb_gf[kMaxDet] = {};  // mixed-precision copies over the bins' span
  RbBinF* rb_bx = nullptr;
  // multi-banding
  int multiband = 0;
  int64_t mb_points = 0;
  double* mb_freq = nullptr;
  double4* mb_pow = nullptr;
  double2* mb_lin[kMaxDet] = {};
  double* mb_quad[kMaxDet] = {};
  int mb_bands = 0;
  int64_t* mb_band_start = nullptr;
  double* mb_band_df = nullptr;
  float2* mb_basis = nullptr;
  float2* mb_lw[kMaxDet] = {};
  double* mb_l2prefix[kMaxDet] = {};
  double mb_lw_scale[kMaxDet] = {};
  double* mb_qprefix[kMaxDet] = {};
  int mb_tm = 0;  // multi-banding time-marginalisation tables set for these bands
  int64_t mb_tm_n = 0;
  double mb_tm_delta_tc = 0.0, mb_tm_antenna_time = 0.0;
  int32_t* mb_tm_ptr = nullptr;
  int32_t* mb_tm_src = nullptr;
  // multi-banding with the IFFT-FFT <h|h>: per band b >= 1 its transform's
  // parameters (pointers into the tables below), the slab of odd-bin parts
  // and, for transforms too long for shared memory, one global slot per CTA
  int mb_fft = 0;
  std::vector<int64_t> mb_band_start_h;
  std::vector<MbFftBand> mbf_bands;
  double* mbf_sqrtw = nullptr;
  double* mbf_odd[kMaxDet] = {};
  double2* mbf_tw = nullptr;
  int mbf_log2m_max = 0;
  double* d_mbf_hh = nullptr;
  size_t mbf_hh_count = 0;
  double2* d_mbf_scratch = nullptr;
  size_t mbf_scratch_count = 0;  // double2 elements
  int64_t mbf_slots = 0;
  // mixed precision (TaylorF2): float32 twiddles and amplitude table, the
  // error slab and the list of points for the float64 recomputation
  float2* mbf_tw32 = nullptr;
  float2* mbf_odd32[kMaxDet] = {};
  float* mbf_aw = nullptr;
  double mbf_aw_scale = 1.0;
  double* d_mbf_err = nullptr;
  int32_t* d_mbf_list = nullptr;  // [B + 1]: the count, then the listed points
  std::vector<double> mb_freq_h;
  int roq_tm = 0;  // ROQ time-marginalisation grid set for these weights
  int64_t roq_tm_n = 0, roq_tm_chunk = 0, roq_tm_rows = 0;
  double roq_tm_delta_tc = 0.0, roq_tm_antenna_time = 0.0;
  double* roq_tm_times = nullptr;
  // reduced-order quadrature
  int roq = 0;
  int roq_nl = 0, roq_nq = 0;
  int64_t roq_time_start = 0, roq_n_time = 0;
  double roq_dt = 0.0;
  double* roq_fl = nullptr;
  double* roq_fq = nullptr;
  double4* roq_pl = nullptr;
  double4* roq_pq = nullptr;
  double2* roq_wl[kMaxDet] = {};
  double* roq_wq[kMaxDet] = {};
  float2* roq_wl32[kMaxDet] = {};  // float32 copy of roq_wl, nodes zero-padded to roq_nl_pad (mixed time marginalisation)
  float roq_wnorm[kMaxDet][kRoqSplits] = {};  // per node group: largest row norm of roq_wl
  int roq_nl_pad = 0, roq_ks = 0;
  int2* roq_tm_g = nullptr;        // per marginalisation sample: its weight-grid index, floor and fraction
  // mixed ROQ time marginalisation: cuBLAS handle and one chunk's buffers
  cublasHandle_t blas = nullptr;
  float2* d_roq_h32 = nullptr;
  float2* d_roq_d32 = nullptr;
  double* d_roq_hh = nullptr;
  int64_t roq_ws_points = 0;
  // work space
  int chunks_per_group = kChunksPerGroup;  // split-K depth of the TaylorF2 mixed kernel (gwl_autotune)
  int64_t ws_B = 0;
  double* d_params = nullptr;
  double* d_out = nullptr;
  PointRec* d_rec = nullptr;
  double* d_part = nullptr;
  size_t part_bytes = 0;
  int32_t* d_order = nullptr;       // [ws_B] point ordering of the mixed TaylorF2 kernel
  int32_t* d_order_hist = nullptr;  // [4 * kOrderMaxKeys + 1]: bucket counts and cursors, then the marked count
  int* last_rf_count = nullptr;     // marked points of the last mixed TaylorF2 evaluation (device)
  double* d_tm = nullptr;
  size_t tm_bytes = 0;
  double* d_twpart = nullptr;  // windowed float64 recomputation: shares, then the per-point unit counters
  size_t twpart_bytes = 0;
  double* h_params = nullptr;  // pinned staging for gwl_eval_host
  double* h_out = nullptr;      // [ws_B + 1]: the results, then the device status word
  int* d_status = nullptr;
  cudaStream_t stream = nullptr;
  SideStream side;  // the accurate kernel beside the fast one
  size_t resident = 0;
  // optional CUDA events around the dominant kernel of each evaluation
  int profiling = 0;
  cudaEvent_t ev_begin = nullptr, ev_end = nullptr;
  int ev_pending = 0;
  std::vector<void*> tables;  // everything allocated for the tables
  std::vector<double> h_freq;  // host copy of the frequency array
  std::mutex mu;
};

namespace {

template <class T>
int dev_alloc(gwl_analysis* a, T** p, size_t count, bool table = true) {
  if (count == 0) count = 1;
  cudaError_t e = cudaMalloc(reinterpret_cast<void**>(p), count * sizeof(T));
  if (e != cudaSuccess) {
    set_error(std::string("cudaMalloc of ") + std::to_string(count * sizeof(T)) + " bytes: " + cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? GWL_ERR_MEMORY : GWL_ERR_CUDA;
  }
  if (table) {
    a->tables.push_back(*p);
    a->resident += count * sizeof(T);
  }
  return GWL_OK;
}

template <class T>
int upload(gwl_analysis* a, T** dst, const std::vector<T>& src) {
  int rc = dev_alloc(a, dst, src.size());
  if (rc) return rc;
  GWL_CUDA(cudaMemcpy(*dst, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice));
  return GWL_OK;
}

void free_workspace(gwl_analysis* a) {
  cudaFree(a->d_params);
  cudaFree(a->d_out);
  cudaFree(a->d_rec);
  cudaFree(a->d_part);
  cudaFree(a->d_order);
  cudaFree(a->d_order_hist);
  cudaFree(a->d_tm);
  cudaFree(a->d_twpart);
  a->d_twpart = nullptr;
  a->twpart_bytes = 0;
  cudaFreeHost(a->h_params);
  cudaFreeHost(a->h_out);
  a->h_params = a->h_out = nullptr;
  a->d_params = a->d_out = a->d_part = a->d_tm = nullptr;
  a->d_rec = nullptr;
  a->d_order = a->d_order_hist = nullptr;
  a->last_rf_count = nullptr;
  a->ws_B = 0;
  a->part_bytes = a->tm_bytes = 0;
  cudaFree(a->d_roq_h32);
  cudaFree(a->d_roq_d32);
  cudaFree(a->d_roq_hh);
  a->d_roq_h32 = a->d_roq_d32 = nullptr;
  a->d_roq_hh = nullptr;
  a->roq_ws_points = 0;
  cudaFree(a->d_mbf_hh);
  cudaFree(a->d_mbf_scratch);
  cudaFree(a->d_mbf_err);
  cudaFree(a->d_mbf_list);
  a->d_mbf_hh = nullptr;
  a->d_mbf_scratch = nullptr;
  a->d_mbf_err = nullptr;
  a->d_mbf_list = nullptr;
  a->mbf_hh_count = a->mbf_scratch_count = 0;
  a->mbf_slots = 0;
}

float2 split_ff(double x) {
  const float hi = (float)x;
  const float lo = (float)(x - (double)hi);
  return make_float2(hi, lo);
}

// n-th derivative of f^alpha
double dpow(double f, double alpha, int n) {
  double c = 1.0;
  for (int i = 0; i < n; ++i) c *= (alpha - i);
  return c * std::pow(f, alpha - n);
}

// n-th derivative of ln f
double dlog(double f, int n) {
  if (n == 0) return std::log(f);
  double c = ((n - 1) % 2 == 0) ? 1.0 : -1.0;
  for (int i = 1; i < n; ++i) c *= i;
  return c * std::pow(f, -(double)n);
}

// Taylor coefficients in the bin index of the eight TaylorF2 phase basis
// functions (f^-5/3, f^-1, f^-2/3, f^-1/3, ln f, f^1/3, f^1/3 ln f, f^2/3)
// at frequency f: T[n][b] = phi_b^(n)(f) * df^n / n!.
void basis_taylor(double f, double df, double T[kAnchorOrders][kNumBasis]) {
  double fact = 1.0, dfn = 1.0;
  for (int n = 0; n < kAnchorOrders; ++n) {
    if (n > 0) {
      fact *= n;
      dfn *= df;
    }
    const double s = dfn / fact;
    T[n][0] = dpow(f, -5.0 / 3.0, n) * s;
    T[n][1] = dpow(f, -1.0, n) * s;
    T[n][2] = dpow(f, -2.0 / 3.0, n) * s;
    T[n][3] = dpow(f, -1.0 / 3.0, n) * s;
    T[n][4] = dlog(f, n) * s;
    T[n][5] = dpow(f, 1.0 / 3.0, n) * s;
    double leib = 0.0, binom = 1.0;  // Leibniz rule for f^1/3 ln f
    for (int i = 0; i <= n; ++i) {
      if (i > 0) binom = binom * (n - i + 1) / i;
      leib += binom * dpow(f, 1.0 / 3.0, n - i) * dlog(f, i);
    }
    T[n][6] = leib * s;
    T[n][7] = dpow(f, 2.0 / 3.0, n) * s;
  }
}

int g_sm_count = 0;

int sm_count() {
  if (g_sm_count == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&g_sm_count, cudaDevAttrMultiProcessorCount, dev);
    if (g_sm_count <= 0) g_sm_count = 152;
  }
  return g_sm_count;
}

LaunchArgs make_args(gwl_analysis* a, int64_t B, int precision) {
  LaunchArgs L;
  std::memset(&L, 0, sizeof(L));
  L.model = a->model;
  L.n_det = a->n_det;
  L.precision = precision;
  // real-part partials suffice unless |<d|h>| (phase marginalisation) is needed
  L.cplx = (precision == GWL_PRECISION_MIXED && a->model == GWL_MODEL_TAYLORF2) ? (a->phase_marg || a->time_marg) : 1;
  L.B = B;
  L.n_bins = a->n_bins;
  L.k_lo = a->k_lo;
  L.k_hi = a->k_hi;
  L.k_base = a->k_base;
  L.chunk = precision == GWL_PRECISION_FP64 ? kChunkPlain : kChunkMixed;
  L.n_chunks = precision == GWL_PRECISION_FP64 ? a->n_chunks_plain : a->n_chunks_mixed;
  L.n_groups = L.n_chunks;
  if (precision == GWL_PRECISION_MIXED && a->model == GWL_MODEL_TAYLORF2) {
    // split-K: each CTA walks a strided set of chunks;
    // a fixed number of chunks per group, so that the summation order of a
    // point (and so its result) is the same for every batch size
    L.n_groups = (a->n_chunks_mixed + a->chunks_per_group - 1) / a->chunks_per_group;
  }
  L.duration = a->duration;
  L.step = a->step;
  L.fmin = a->fmin;
  L.k_fmin = a->k_fmin;
  for (int d = 0; d < a->n_det; ++d) {
    L.det[d] = a->geom[d];
    L.strain[d] = a->strain[d];
    L.inv_psd[d] = a->inv_psd[d];
    L.w[d] = a->w[d];
    L.wp[d] = a->wp[d];
    L.wq[d] = a->wq[d];
    L.v[d] = a->v[d];
    L.v_lo[d] = a->v_lo[d];
    L.hh_prefix[d] = a->hh_prefix[d];
    L.rf_p2[d] = a->rf_p2[d];
    L.rf_p1[d] = a->rf_p1[d];
    L.w_scale[d] = a->w_scale[d];
    L.v_scale[d] = a->v_scale[d];
  }
  // the list and its count are set by the entry point that launches k_refine
  L.rf_tol = precision == GWL_PRECISION_MIXED ? a->refine_tol : 0.0;
  L.cos_tab = a->cos_tab;
  L.freq = a->freq;
  L.freq_f = a->freq_f;
  L.basis = a->basis;
  L.ftab = a->ftab;
  L.anchors = a->anchors;
  L.n_anchors = a->n_anchors;
  L.status = a->d_status;
  L.time_marg = a->time_marg;
  L.phase_marg = a->phase_marg;
  L.dist_marg = a->dist_marg;
  L.dist_slope = a->dist_marg && !a->time_marg ? a->dist_slope : 1.0;
  L.jitter = a->jitter;
  L.t_min = a->t_min;
  L.t_max = a->t_max;
  L.delta_tc = 2.0 / a->fs;
  L.start_time0 = a->start0;
  L.n_fft = a->n_bins - 1;
  L.tm_first = 1;
  if (a->multiband && a->mb_tm) {
    // multiband.py:714-726: FFT length Nbs[-1] / 2, times start + j delta_tc,
    // antenna patterns at the prior's mid time
    L.n_fft = a->mb_tm_n;
    L.delta_tc = a->mb_tm_delta_tc;
    L.tm_first = 0;
    L.antenna_fixed = 1;
    L.antenna_time = a->mb_tm_antenna_time;
    L.mb_tm = 1;
    L.mb_tm_ptr = a->mb_tm_ptr;
    L.mb_tm_src = a->mb_tm_src;
  }
  L.tx = a->tx;
  L.ty = a->ty;
  L.tc = a->tc;
  L.tx_f = a->tx_f;
  L.ty_f = a->ty_f;
  L.tc_f = a->tc_f;
  L.nx = a->nx;
  L.ny = a->ny;
  for (int q = 0; q < 4; ++q) L.bbox[q] = a->bbox[q];
  {
    // the x bounds as float32 that give the same test of a float32 x:
    // bbox[0] rounded up, bbox[1] rounded down
    float lo = (float)a->bbox[0], hi = (float)a->bbox[1];
    if ((double)lo < a->bbox[0]) lo = std::nextafter(lo, INFINITY);
    if ((double)hi > a->bbox[1]) hi = std::nextafter(hi, -INFINITY);
    L.bbox_x_f[0] = lo;
    L.bbox_x_f[1] = hi;
  }
  L.ref_dist = a->ref_dist;
  L.tm_step = a->duration / (double)(a->n_bins - 1);  // linspace(0, T, L + 1) spacing, L = n_bins - 1
  L.tm_inv_step = (double)(a->n_bins - 1) / a->duration;
  L.tm_prob = a->t_max > a->t_min ? 1.0 / (a->t_max - a->t_min) : 0.0;
  L.tm_prior = a->tm_prior;
  L.tm_prior_f = a->tm_prior_f;
  L.tm_prior_n = a->tm_prior_n;
  L.tm_prior_t0 = a->tm_prior_t0;
  L.tm_prior_inv_h = a->tm_prior_inv_h;
  L.inv_ref_dist = a->ref_dist > 0 ? 1.0 / a->ref_dist : 0.0;
  L.relbin = a->relbin;
  L.rb_edges = a->rb_edges;
  L.rb_index = a->rb_index;
  L.rb_freq = a->rb_freq;
  L.rb_bin = a->rb_bin;
  L.rb_bx = a->rb_bx;
  for (int d = 0; d < a->n_det; ++d) {
    L.rb_h0inv[d] = a->rb_h0inv[d];
    L.rb_sum[d] = a->rb_sum[d];
    L.rb_g[d] = a->rb_g[d];
    L.rb_gf[d] = a->rb_gf[d];
  }
  L.multiband = a->multiband;
  L.mb_points = a->mb_points;
  L.mb_freq = a->mb_freq;
  L.mb_pow = a->mb_pow;
  for (int d = 0; d < a->n_det; ++d) {
    L.mb_lin[d] = a->mb_lin[d];
    L.mb_quad[d] = a->mb_quad[d];
  }
  L.mb_bands = a->mb_bands;
  L.mb_band_start = a->mb_band_start;
  L.mb_band_df = a->mb_band_df;
  L.mb_basis = a->mb_basis;
  for (int d = 0; d < a->n_det; ++d) {
    L.mb_lw[d] = a->mb_lw[d];
    L.mb_l2prefix[d] = a->mb_l2prefix[d];
    L.mb_lw_scale[d] = a->mb_lw_scale[d];
    L.mb_qprefix[d] = a->mb_qprefix[d];
  }
  L.roq = a->roq;
  L.roq_nl = a->roq_nl;
  L.roq_nq = a->roq_nq;
  L.roq_time_start = a->roq_time_start;
  L.roq_n_time = a->roq_n_time;
  L.roq_dt = a->roq_dt;
  L.roq_fl = a->roq_fl;
  L.roq_fq = a->roq_fq;
  L.roq_pl = a->roq_pl;
  L.roq_pq = a->roq_pq;
  for (int d = 0; d < a->n_det; ++d) {
    L.roq_wl[d] = a->roq_wl[d];
    L.roq_wq[d] = a->roq_wq[d];
    L.roq_wl32[d] = a->roq_wl32[d];
    for (int sp = 0; sp < kRoqSplits; ++sp) L.roq_wnorm[d][sp] = a->roq_wnorm[d][sp];
  }
  L.roq_nl_pad = a->roq_nl_pad;
  L.roq_ks = a->roq_ks;
  L.roq_tm_g = a->roq_tm_g;
  if (a->roq && a->roq_tm) {
    // roq.py:320-331: the marginalisation's own time grid, antenna patterns
    // and delays at the prior's mid time
    L.roq_tm = 1;
    L.roq_tm_n = a->roq_tm_n;
    L.roq_tm_chunk = a->roq_tm_chunk;
    L.roq_tm_rows = a->roq_tm_rows;
    L.roq_tm_times = a->roq_tm_times;
    L.delta_tc = a->roq_tm_delta_tc;
    L.antenna_fixed = 1;
    L.antenna_time = a->roq_tm_antenna_time;
  }
  return L;
}

int ensure_workspace(gwl_analysis* a, int64_t B, const LaunchArgs& L) {
  const size_t part = (size_t)std::max(a->n_chunks_plain, a->n_chunks_mixed) * B * a->n_det * kPartStride *
                      sizeof(double);
  size_t tm = 0;
  if (a->time_marg && !a->roq) {  // ROQ marginalises without an FFT
    // the float64 kernel over the whole FFT keeps one transform per resident
    // CTA in global memory; the windowed kernels need none
    LaunchArgs F = L;
    F.precision = GWL_PRECISION_FP64;
    if (!time_marg_window_fits(F)) tm = time_marg_work_bytes(L);
    // the mixed windowed multi-banding kernel: one slot of banded values per CTA
    if (a->multiband && a->mb_tm && a->model == GWL_MODEL_TAYLORF2)
      tm = std::max(tm, (size_t)time_marg_window_slots() * (size_t)a->mb_points * sizeof(float2));
  }
  if (B <= a->ws_B && part <= a->part_bytes && tm <= a->tm_bytes) return GWL_OK;
  GWL_CUDA(cudaStreamSynchronize(a->stream));
  free_workspace(a);
  int rc;
  if ((rc = dev_alloc(a, &a->d_params, (size_t)GWL_NPARAM * B, false))) return rc;
  if ((rc = dev_alloc(a, &a->d_out, (size_t)B, false))) return rc;
  if ((rc = dev_alloc(a, &a->d_rec, (size_t)B, false))) return rc;
  if ((rc = dev_alloc(a, &a->d_part, part / sizeof(double), false))) return rc;
  if ((rc = dev_alloc(a, &a->d_order, (size_t)B, false))) return rc;
  if ((rc = dev_alloc(a, &a->d_order_hist, (size_t)4 * kOrderMaxKeys + 1, false))) return rc;
  if (tm) {
    if ((rc = dev_alloc(a, reinterpret_cast<char**>(&a->d_tm), tm, false))) return rc;
  }
  GWL_CUDA(cudaMallocHost(&a->h_params, sizeof(double) * GWL_NPARAM * B));
  GWL_CUDA(cudaMallocHost(&a->h_out, sizeof(double) * (B + 1)));
  a->ws_B = B;
  a->part_bytes = part;
  a->tm_bytes = tm;
  return GWL_OK;
}

// The windowed time-marginalisation kernels' float64 recomputation: shares
// of at most kShareUnits units (window sums and <h|h>), then one finished-unit
// counter per unit; grown on demand.
constexpr int64_t kShareUnits = 4096;

int ensure_window_shares(gwl_analysis* a, const LaunchArgs& L, cudaStream_t s, size_t* share) {
  *share = time_marg_window_share_bytes(L);
  const size_t total = *share * kShareUnits + sizeof(int) * kShareUnits;
  if (total <= a->twpart_bytes) return GWL_OK;
  GWL_CUDA(cudaStreamSynchronize(s));
  cudaFree(a->d_twpart);
  a->d_twpart = nullptr;
  a->twpart_bytes = 0;
  int rc = dev_alloc(a, reinterpret_cast<char**>(&a->d_twpart), total, false);
  if (rc) return rc;
  a->twpart_bytes = total;
  return GWL_OK;
}

// Marks of a mixed time-marginalised kernel (after the prologue, which would
// otherwise apply the full-grid kernels' bound): listed in d_order, counted
// in d_order_hist.
int set_window_marks(gwl_analysis* a, LaunchArgs& L, cudaStream_t s) {
  L.rf_tol = a->refine_tol;
  L.rf_count = a->d_order_hist;
  L.rf_list = a->d_order;
  a->last_rf_count = L.rf_count;
  GWL_CUDA(cudaMemsetAsync(L.rf_count, 0, sizeof(int32_t), s));
  return GWL_OK;
}

// The float64 recomputation of the listed points by the windowed kernel,
// split over several CTAs per point.
int launch_window_refine(gwl_analysis* a, const LaunchArgs& L, cudaStream_t s, size_t share) {
  LaunchArgs R = L;
  R.precision = GWL_PRECISION_FP64;
  R.rf_tol = 0.0;
  R.tw_refine_only = 1;
  R.tw_part = a->d_twpart;
  R.tw_part_units = kShareUnits;
  R.tw_done = reinterpret_cast<int*>(reinterpret_cast<char*>(a->d_twpart) + share * kShareUnits);
  GWL_CUDA(cudaMemsetAsync(R.tw_done, 0, sizeof(int) * kShareUnits, s));
  GWL_CUDA(launch_time_marg_window(R, s));
  return GWL_OK;
}

// The windowed kernel after the prologue: mixed precision with its marks and
// their recomputation, or float64 alone.
int launch_window_marg(gwl_analysis* a, LaunchArgs& L, cudaStream_t s, bool mixed, size_t share) {
  int rc;
  if (mixed && (rc = set_window_marks(a, L, s))) return rc;
  GWL_CUDA(launch_time_marg_window(L, s));
  if (mixed && (rc = launch_window_refine(a, L, s, share))) return rc;
  return GWL_OK;
}

// ROQ with time marginalisation in mixed precision, chunk by chunk: the node
// values, one complex float32 GEMM per detector (D_d = W_d^T conj(h_d) over
// every weight row), the interpolation and marginalisation with the error
// bound, then the float64 kernel on the listed points.
int run_roq_tm_mixed(gwl_analysis* a, LaunchArgs& L, cudaStream_t s) {
  const int64_t B = L.B, chunk = std::min<int64_t>(B, kRoqMixedChunk);
  const int64_t np = a->roq_nl_pad, ks = a->roq_ks, nt = a->roq_n_time, D = a->n_det;
  if (np > INT32_MAX || nt * chunk > INT32_MAX) {
    set_error("ROQ time marginalisation: too many nodes or weight rows for a matrix product");
    return GWL_ERR_UNSUPPORTED;
  }
  int rc;
  if (a->roq_ws_points < chunk) {
    cudaFree(a->d_roq_h32);
    cudaFree(a->d_roq_d32);
    cudaFree(a->d_roq_hh);
    a->d_roq_h32 = a->d_roq_d32 = nullptr;
    a->d_roq_hh = nullptr;
    a->roq_ws_points = 0;
    if ((rc = dev_alloc(a, &a->d_roq_h32, (size_t)(D * chunk * np), false))) return rc;
    if ((rc = dev_alloc(a, &a->d_roq_d32, (size_t)(D * kRoqSplits * chunk * nt), false))) return rc;
    if ((rc = dev_alloc(a, &a->d_roq_hh, (size_t)chunk, false))) return rc;
    a->roq_ws_points = chunk;
  }
  if (!a->blas) {
    if (cublasCreate(&a->blas) != CUBLAS_STATUS_SUCCESS) {
      a->blas = nullptr;
      set_error("cublasCreate failed");
      return GWL_ERR_CUDA;
    }
    // float32 arithmetic throughout: no reduced-precision tensor-core path
    cublasSetMathMode(a->blas, CUBLAS_PEDANTIC_MATH);
  }
  if (cublasSetStream(a->blas, s) != CUBLAS_STATUS_SUCCESS) {
    set_error("cublasSetStream failed");
    return GWL_ERR_CUDA;
  }
  const bool marks = a->refine_tol > 0;
  L.rf_tol = a->refine_tol;
  L.rf_count = marks ? a->d_order_hist : nullptr;
  L.rf_list = marks ? a->d_order : nullptr;
  if (marks) GWL_CUDA(cudaMemsetAsync(L.rf_count, 0, sizeof(int32_t), s));
  L.roq_h32 = a->d_roq_h32;
  L.roq_d32 = a->d_roq_d32;
  L.roq_hh = a->d_roq_hh;
  const cuComplex one = make_cuComplex(1.f, 0.f), zero = make_cuComplex(0.f, 0.f);
  for (int64_t c0 = 0; c0 < B; c0 += chunk) {
    const int64_t cn = std::min(chunk, B - c0);
    L.roq_c0 = c0;
    L.roq_cn = cn;
    GWL_CUDA(launch_roq_nodes32(L, s));
    for (int64_t d = 0; d < D; ++d) {
      // column-major, one batch entry per node group s: W_d,s^T (nt x ks, the
      // row-major [nt][np] table from column s ks), H_d,s (ks x cn), D_d,s (nt x cn)
      const cublasStatus_t st = cublasCgemmStridedBatched(
          a->blas, CUBLAS_OP_T, CUBLAS_OP_N, (int)nt, (int)cn, (int)ks, &one,
          reinterpret_cast<const cuComplex*>(a->roq_wl32[d]), (int)np, (long long)ks,
          reinterpret_cast<const cuComplex*>(a->d_roq_h32 + (size_t)(d * cn * np)), (int)np, (long long)ks, &zero,
          reinterpret_cast<cuComplex*>(a->d_roq_d32 + (size_t)(d * kRoqSplits * cn * nt)), (int)nt,
          (long long)(cn * nt), kRoqSplits);
      if (st != CUBLAS_STATUS_SUCCESS) {
        set_error("cublasCgemmStridedBatched failed with status " + std::to_string((int)st));
        return GWL_ERR_CUDA;
      }
    }
    GWL_CUDA(launch_roq_tm_mixed(L, s));
  }
  if (marks) {
    LaunchArgs R = L;
    R.rf_tol = 0.0;
    R.rf_list_only = 1;
    GWL_CUDA(launch_roq_time_marginalized(R, s));
    a->last_rf_count = L.rf_count;
  }
  return GWL_OK;
}

// An NVTX range over a scope (a no-op unless a profiler is attached): the
// entry points mark their launch sequences, the host paths also their
// copies.
struct TraceRange {
  explicit TraceRange(const char* name) { nvtxRangePushA(name); }
  ~TraceRange() { nvtxRangePop(); }
  TraceRange(const TraceRange&) = delete;
  TraceRange& operator=(const TraceRange&) = delete;
};

// Multi-banding with the IFFT-FFT <h|h>: the odd-bin transforms of every band
// b >= 1 into the slab that the multi-banding kernels add to <h|h>.  Mixed
// precision with TaylorF2: float32 transforms with an error bound, then the
// float64 kernel over the points whose bound exceeds the tolerance.  The
// bound holds for lnL = f(<d|h>) - <h|h> / 2 (no marginalisation, phase, time),
// whose slope in <h|h> is -1/2; with the distance table the slope is
// -E[(d_ref / d)^2] / 2, unbounded by the tolerance's terms, so distance
// marginalisation keeps the float64 transforms.
int run_mb_fft(gwl_analysis* a, LaunchArgs& L, cudaStream_t s) {
  const bool mixed = L.precision == GWL_PRECISION_MIXED && a->model == GWL_MODEL_TAYLORF2 && !a->dist_marg;
  const size_t need = (size_t)a->mb_bands * a->n_det * L.B;
  bool glob = false;
  for (const MbFftBand& bd : a->mbf_bands)
    glob = glob || !bd.in_smem || (mixed && !mb_hh_fft32_in_smem(bd.log2m));
  // one global slot per resident CTA (two per SM for the float32 kernel)
  const int64_t slots = glob ? (int64_t)(mixed ? 2 : 1) * sm_count() : 0;
  const size_t scratch = glob ? ((size_t)slots << a->mbf_log2m_max) : 0;  // double2 elements
  if (need > a->mbf_hh_count || scratch > a->mbf_scratch_count) {
    GWL_CUDA(cudaStreamSynchronize(s));
    int rc;
    if (need > a->mbf_hh_count) {
      cudaFree(a->d_mbf_hh);
      cudaFree(a->d_mbf_err);
      cudaFree(a->d_mbf_list);
      a->d_mbf_hh = a->d_mbf_err = nullptr;
      a->d_mbf_list = nullptr;
      a->mbf_hh_count = 0;
      if ((rc = dev_alloc(a, &a->d_mbf_hh, need, false))) return rc;
      if ((rc = dev_alloc(a, &a->d_mbf_err, need, false))) return rc;
      if ((rc = dev_alloc(a, &a->d_mbf_list, (size_t)L.B + 1, false))) return rc;
      a->mbf_hh_count = need;
    }
    if (scratch > a->mbf_scratch_count) {
      cudaFree(a->d_mbf_scratch);
      a->d_mbf_scratch = nullptr;
      a->mbf_scratch_count = 0;
      if ((rc = dev_alloc(a, &a->d_mbf_scratch, scratch, false))) return rc;
      a->mbf_scratch_count = scratch;
    }
  }
  a->mbf_slots = glob ? slots : 0;
  if (!mixed) {
    for (MbFftBand bd : a->mbf_bands) {
      bd.out = a->d_mbf_hh;
      GWL_CUDA(launch_mb_hh_fft(L, bd, a->d_mbf_scratch, a->mbf_slots, false, s));
    }
  } else {
    for (MbFftBand bd : a->mbf_bands) {
      bd.out = a->d_mbf_hh;
      bd.err = a->d_mbf_err;
      bd.in_smem = mb_hh_fft32_in_smem(bd.log2m);
      GWL_CUDA(launch_mb_hh_fft(L, bd, a->d_mbf_scratch, a->mbf_slots, true, s));
    }
    if (a->refine_tol > 0) {
      int32_t* count = a->d_mbf_list;
      GWL_CUDA(cudaMemsetAsync(count, 0, sizeof(int32_t), s));
      GWL_CUDA(launch_mb_fft_marks(L, a->d_mbf_err, a->refine_tol, count + 1, count, s));
      for (MbFftBand bd : a->mbf_bands) {
        bd.out = a->d_mbf_hh;
        bd.list = count + 1;
        bd.list_count = count;
        GWL_CUDA(launch_mb_hh_fft(L, bd, a->d_mbf_scratch, a->mbf_slots, false, s));
      }
    }
  }
  L.mb_fft_hh = a->d_mbf_hh;
  return GWL_OK;
}

int run_eval(gwl_analysis* a, const double* d_params, int64_t B, int precision, double* d_out, double* d_dh,
             double* d_hh, cudaStream_t s, double* d_series = nullptr) {
  if (precision != GWL_PRECISION_FP64 && precision != GWL_PRECISION_MIXED) {
    set_error("precision must be GWL_PRECISION_FP64 or GWL_PRECISION_MIXED");
    return GWL_ERR_ARGUMENT;
  }
  if (B <= 0) return GWL_OK;
  LaunchArgs L = make_args(a, B, precision);
  L.tm_series = d_series;
  int rc = ensure_workspace(a, B, L);
  if (rc) return rc;
  L.params = d_params;
  L.rec = a->d_rec;
  L.part = a->d_part;
  L.out = d_out;
  L.dh_out = d_dh;
  L.hh_out = d_hh;
  L.tm_work = a->d_tm;
  L.tm_series = d_series;
  if (a->multiband && a->mb_points > 0) {
    L.tw_scratch = reinterpret_cast<float2*>(a->d_tm);
    L.tw_scratch_slots = std::min<int64_t>(time_marg_window_slots(),
                                           (int64_t)(a->tm_bytes / ((size_t)a->mb_points * sizeof(float2))));
  }
  if (a->roq && a->time_marg && d_out) {
    if (!a->roq_tm) {
      set_error("ROQ with time marginalisation needs gwl_set_roq_time_marginalization");
      return GWL_ERR_ARGUMENT;
    }
    // mixed precision: float32 matrix products and marginalisation, the
    // points over the error bound recomputed in float64; float64 alone when
    // the time series is requested
    const bool mixed = precision == GWL_PRECISION_MIXED && !d_series && roq_tm_mixed_fits(L);
    L.precision = GWL_PRECISION_FP64;
    L.rf_tol = 0.0;
    a->last_rf_count = nullptr;
    GWL_CUDA(launch_prologue(L, s));
    if (a->profiling) GWL_CUDA(cudaEventRecord(a->ev_begin, s));
    if (mixed) {
      if ((rc = run_roq_tm_mixed(a, L, s))) return rc;
    } else {
      GWL_CUDA(launch_roq_time_marginalized(L, s));
    }
    if (a->profiling) {
      GWL_CUDA(cudaEventRecord(a->ev_end, s));
      a->ev_pending = 1;
    }
    return GWL_OK;
  }
  if ((a->relbin || a->multiband) && a->time_marg && d_out) {
    // relative binning / multi-banding with time marginalisation: the float64
    // time-marginalised kernel over the rebuilt full-resolution integrand
    if (a->relbin && !a->rb_tm) {
      set_error("relative binning with time marginalisation needs gwl_set_relative_binning_time_weights");
      return GWL_ERR_ARGUMENT;
    }
    if (a->multiband && !a->mb_tm) {
      set_error("multi-banding with time marginalisation needs gwl_set_multiband_time_marginalization");
      return GWL_ERR_ARGUMENT;
    }
    // the windowed four-step transform where its shared memory fits (mixed
    // precision for relative binning and TaylorF2 multi-banding, with the
    // float64 kernel recomputing the points over the tolerance), else the
    // float64 kernel over the whole FFT
    L.rf_tol = 0.0;
    L.precision = (precision == GWL_PRECISION_MIXED && (a->relbin || a->model == GWL_MODEL_TAYLORF2))
                      ? GWL_PRECISION_MIXED
                      : GWL_PRECISION_FP64;
    bool window = time_marg_window_fits(L) && (L.precision != GWL_PRECISION_MIXED || time_marg_window_mixed_ready(L));
    if (!window && L.precision == GWL_PRECISION_MIXED) {
      L.precision = GWL_PRECISION_FP64;
      window = time_marg_window_fits(L);
    }
    const bool mixed = window && L.precision == GWL_PRECISION_MIXED && a->refine_tol > 0;
    size_t share = 0;
    a->last_rf_count = nullptr;  // no marks unless the mixed kernel sets them
    if (mixed && (rc = ensure_window_shares(a, L, s, &share))) return rc;
    GWL_CUDA(launch_prologue(L, s));
    if (a->profiling) GWL_CUDA(cudaEventRecord(a->ev_begin, s));
    if (a->multiband && a->mb_fft && (rc = run_mb_fft(a, L, s))) return rc;
    if (window) {
      if ((rc = launch_window_marg(a, L, s, mixed, share))) return rc;
    } else {
      GWL_CUDA(launch_time_marginalized(L, s));
    }
    if (a->profiling) {
      GWL_CUDA(cudaEventRecord(a->ev_end, s));
      a->ev_pending = 1;
    }
    return GWL_OK;
  }
  if (a->relbin || a->multiband || a->roq) {
    // relative binning / multi-banding / ROQ: per-point set-up, then one warp
    // per point over the bin edges, banded frequencies or nodes (no marking
    // for the accurate kernel: it serves the full-grid TaylorF2 kernels)
    L.rf_tol = 0.0;
    GWL_CUDA(launch_prologue(L, s));
    if (a->profiling) GWL_CUDA(cudaEventRecord(a->ev_begin, s));
    if (a->multiband && a->mb_fft && (rc = run_mb_fft(a, L, s))) return rc;
    if (a->relbin) {
      GWL_CUDA(launch_relbin(L, s));
    } else if (a->multiband) {
      if (precision == GWL_PRECISION_MIXED && a->model == GWL_MODEL_TAYLORF2) {
        // points whose error bound exceeds the tolerance are marked by the
        // mixed kernel and recomputed by the float64 one
        L.rf_tol = a->refine_tol;
        if (L.rf_tol > 0) {
          L.rf_count = a->d_order_hist;
          a->last_rf_count = L.rf_count;
          GWL_CUDA(cudaMemsetAsync(L.rf_count, 0, sizeof(int32_t), s));
        }
        GWL_CUDA(launch_multiband_mixed(L, s));
        if (L.rf_tol > 0) {
          LaunchArgs R = L;
          R.precision = GWL_PRECISION_FP64;
          R.mb_refine_only = 1;
          GWL_CUDA(launch_multiband(R, s));
        }
      } else {
        GWL_CUDA(launch_multiband(L, s));
      }
    } else {
      GWL_CUDA(launch_roq(L, s));
    }
    if (a->profiling) {
      GWL_CUDA(cudaEventRecord(a->ev_end, s));
      a->ev_pending = 1;
    }
    return GWL_OK;
  }
  if (d_dh) L.cplx = 1;  // complex <d|h> requested
  const bool ordered = precision == GWL_PRECISION_MIXED && a->model == GWL_MODEL_TAYLORF2 && !(a->time_marg && d_out);
  if (ordered) {
    // group the points by band end (see LaunchArgs::order)
    L.order = a->d_order;
    L.order_hist = a->d_order_hist;
    if (a->time_marg && d_out) L.rf_tol = 0.0;  // the time-marginalised kernel has its own integrand
    ordering_with_marks(L);
    a->last_rf_count = L.rf_count;
    GWL_CUDA(cudaMemsetAsync(L.order_hist, 0, sizeof(int32_t) * (2 * L.order_keys + 1), s));
  } else if (precision == GWL_PRECISION_MIXED && a->model == GWL_MODEL_SINEGAUSSIAN && !(a->time_marg && d_out)) {
    // sine-Gaussian: points ordered by centre frequency; the finalize marks
    // the points whose error bound exceeds the tolerance and counts them
    // after the histogram; k_sg_refine recomputes them
    L.order = a->d_order;
    L.order_hist = a->d_order_hist;
    ordering_by_peak(L);
    if (!(L.rf_tol > 0)) L.rf_count = nullptr;
    a->last_rf_count = L.rf_count;
    GWL_CUDA(cudaMemsetAsync(L.order_hist, 0, sizeof(int32_t) * (2 * L.order_keys + 1), s));
  } else {
    L.rf_tol = 0.0;
  }
  GWL_CUDA(launch_prologue(L, s));
  if (ordered || L.order) GWL_CUDA(launch_order(L, s));
  if (a->profiling) GWL_CUDA(cudaEventRecord(a->ev_begin, s));
  if (a->time_marg && d_out) {
    // mixed TaylorF2: the whole-FFT kernel marks the points over its error
    // bound; the windowed float64 kernel recomputes them, split over CTAs
    const bool marks = precision == GWL_PRECISION_MIXED && a->model == GWL_MODEL_TAYLORF2 && a->refine_tol > 0 &&
                       time_marg_window_refine_fits(L);
    size_t share = 0;
    a->last_rf_count = nullptr;  // no marks unless set below
    if (marks) {
      if ((rc = ensure_window_shares(a, L, s, &share))) return rc;
      set_window_marks(a, L, s);
    }
    if (precision == GWL_PRECISION_MIXED && a->model == GWL_MODEL_SINEGAUSSIAN) {
      // the mixed sine-Gaussian pass first: its float-float <h|h> partial sums
      // are what the time-marginalised kernel reads
      LaunchArgs P = L;
      P.rf_tol = 0.0;
      P.rf_count = nullptr;
      GWL_CUDA(launch_mixed(P, s));
    }
    GWL_CUDA(launch_time_marginalized(L, s));
    if (marks) GWL_CUDA(launch_time_marg_marks(L, s));
    if (marks && (rc = launch_window_refine(a, L, s, share))) return rc;
    if (a->profiling) {
      GWL_CUDA(cudaEventRecord(a->ev_end, s));
      a->ev_pending = 1;
    }
    return GWL_OK;
  }
  const bool acc = precision == GWL_PRECISION_MIXED && a->model == GWL_MODEL_TAYLORF2 && L.rf_tol > 0;
  if (acc) {
    // the marked points in the accurate kernel on the side stream, beside the fast kernel
    GWL_CUDA(side_fork(a->side, s));
    GWL_CUDA(launch_mixed_acc(L, a->side.stream));
  }
  if (precision == GWL_PRECISION_FP64) {
    GWL_CUDA(launch_plain(L, s));
  } else {
    GWL_CUDA(launch_mixed(L, s));
  }
  if (a->profiling) {
    GWL_CUDA(cudaEventRecord(a->ev_end, s));
    a->ev_pending = 1;
  }
  if (acc) GWL_CUDA(side_join(a->side, s));
  GWL_CUDA(launch_finalize(L, s));
  if (precision == GWL_PRECISION_MIXED && a->model == GWL_MODEL_SINEGAUSSIAN && L.rf_tol > 0)
    GWL_CUDA(launch_sg_refine(L, s));
  return GWL_OK;
}

}  // namespace

namespace gwl {

// Launch arguments of a mixed-precision TaylorF2 evaluation of B points for an
// entry point that supplies its own work space; also the bytes it needs for
// the per-point records and the partial sums.  Allocates nothing.
int noalloc_launch_args(gwl_analysis* a, int64_t B, LaunchArgs* L, size_t* rec_bytes, size_t* part_bytes) {
  if (a->model != GWL_MODEL_TAYLORF2 || a->time_marg || a->relbin || a->multiband || a->roq) {
    set_error("the allocation-free entry point serves mixed-precision TaylorF2 analyses without time "
              "marginalisation, relative binning, multi-banding or ROQ");
    return GWL_ERR_UNSUPPORTED;
  }
  *L = make_args(a, B, GWL_PRECISION_MIXED);
  *rec_bytes = (size_t)B * sizeof(PointRec);
  *part_bytes = (size_t)L->n_groups * a->n_det * kPartStride * (size_t)B * sizeof(double);
  return GWL_OK;
}

}  // namespace gwl

// Batches of several analyses in one launch sequence (a persistent kernel per
// detector count), optionally replayed from captured CUDA graphs.
struct gwl_batcher {
  LaunchArgs* d_args = nullptr;
  LaunchArgs* h_args = nullptr;
  int cap_items = 0;
  int64_t* d_off = nullptr;
  int64_t* h_off = nullptr;
  int4* d_units = nullptr;
  int4* h_units = nullptr;
  int64_t cap_units = 0;
  int* d_counter = nullptr;
  PointRec* d_rec = nullptr;
  int64_t cap_points = 0;
  double* d_part = nullptr;
  size_t cap_part = 0;  // doubles
  int32_t* d_order = nullptr;  // [cap_points]
  int32_t* d_hist = nullptr;   // [cap_hist] per item 2 * order_keys
  size_t cap_hist = 0;
  int* d_status = nullptr;
  cudaEvent_t staged = nullptr;
  bool staged_pending = false;
  SideStream side;  // the accurate kernels beside the fast ones
  int use_graphs = 0;
  std::map<std::vector<int64_t>, cudaGraphExec_t> graphs;
  std::mutex mu;
};

namespace {

void drop_graphs(gwl_batcher* b) {
  for (auto& kv : b->graphs) cudaGraphExecDestroy(kv.second);
  b->graphs.clear();
}

template <class T>
int grow(T** dptr, T** hptr, size_t have, size_t need) {
  if (need <= have) return GWL_OK;
  if (dptr) {
    cudaFree(*dptr);
    *dptr = nullptr;
    GWL_CUDA(cudaMalloc(reinterpret_cast<void**>(dptr), need * sizeof(T)));
  }
  if (hptr) {
    cudaFreeHost(*hptr);
    *hptr = nullptr;
    GWL_CUDA(cudaMallocHost(reinterpret_cast<void**>(hptr), need * sizeof(T)));
  }
  return GWL_OK;
}

}  // namespace

extern "C" {

const char* gwl_last_error(void) { return t_last_error.c_str(); }

const char* gwl_version(void) { return "bilby_gb300 gwlnl 0.1 (sm_103a)"; }

int gwl_analysis_create(const gwl_analysis_desc* desc, gwl_analysis** out) {
  if (!desc || !out) {
    set_error("null argument");
    return GWL_ERR_ARGUMENT;
  }
  *out = nullptr;
  if (desc->model != GWL_MODEL_SINEGAUSSIAN && desc->model != GWL_MODEL_TAYLORF2) {
    set_error("unsupported source model");
    return GWL_ERR_UNSUPPORTED;
  }
  if (desc->n_detectors < 1 || desc->n_detectors > kMaxDet || desc->n_bins < 3 || !desc->frequency ||
      !desc->detectors || !(desc->duration > 0) || !(desc->sampling_frequency > 0)) {
    set_error("invalid analysis description (detectors 1..4, n_bins >= 3, positive duration and rate)");
    return GWL_ERR_ARGUMENT;
  }
  auto* a = new gwl_analysis();
  a->model = desc->model;
  a->n_det = desc->n_detectors;
  a->n_bins = desc->n_bins;
  a->duration = desc->duration;
  a->fs = desc->sampling_frequency;
  a->fmin = desc->minimum_frequency;
  const int64_t N = desc->n_bins;
  const double* f = desc->frequency;
  // The kernels take f_k = k * step (bilby's linspace(0, fs/2, N) grid).
  a->step = f[N - 1] / (double)(N - 1);
  for (int64_t k = 0; k < N; ++k) {
    if (std::fabs(f[k] - k * a->step) > 1e-9 * std::max(1.0, f[N - 1])) {
      set_error("frequency_array is not the uniform grid k * df starting at 0");
      delete a;
      return GWL_ERR_UNSUPPORTED;
    }
  }
  // in-band hull over all detectors
  int64_t lo = N, hi = -1;
  for (int d = 0; d < a->n_det; ++d) {
    const gwl_detector& det = desc->detectors[d];
    if (!det.strain || !det.psd || !det.mask) {
      set_error("detector arrays must be non-null");
      delete a;
      return GWL_ERR_ARGUMENT;
    }
    for (int64_t k = 0; k < N; ++k)
      if (det.mask[k]) {
        lo = std::min(lo, k);
        hi = std::max(hi, k);
      }
    std::memcpy(a->geom[d].vertex, det.vertex, sizeof(det.vertex));
    std::memcpy(a->geom[d].tensor, det.tensor, sizeof(det.tensor));
    a->geom[d].start_time = det.start_time;
  }
  if (hi < lo) {
    set_error("frequency masks select no bins");
    delete a;
    return GWL_ERR_ARGUMENT;
  }
  a->start0 = a->geom[0].start_time;
  a->k_lo = lo;
  a->k_hi = hi + 1;
  a->k_base = (lo / kBinAlign) * kBinAlign;
  const int64_t span = a->k_hi - a->k_base;
  a->n_chunks_plain = (span + kChunkPlain - 1) / kChunkPlain;
  a->n_chunks_mixed = (span + kChunkMixed - 1) / kChunkMixed;
  a->n_pad = std::max({N + 1, a->k_base + a->n_chunks_plain * kChunkPlain, a->k_base + a->n_chunks_mixed * kChunkMixed});
  a->n_pad = (a->n_pad + 15) / 16 * 16;
  a->k_fmin = N;
  for (int64_t k = 0; k < N; ++k)
    if (f[k] >= a->fmin) {
      a->k_fmin = k;
      break;
    }
  const int64_t P = a->n_pad;
  int rc = GWL_OK;
  cudaError_t ce = cudaStreamCreateWithFlags(&a->stream, cudaStreamNonBlocking);
  if (ce == cudaSuccess) ce = side_stream_create(&a->side);
  if (ce != cudaSuccess) {
    set_error(std::string("cudaStreamCreate: ") + cudaGetErrorString(ce));
    if (a->stream) cudaStreamDestroy(a->stream);
    side_stream_destroy(&a->side);
    delete a;
    return GWL_ERR_CUDA;
  }
  if ((rc = dev_alloc(a, &a->d_status, 1))) goto fail;
  if (cudaMemset(a->d_status, 0, sizeof(int)) != cudaSuccess) {
    rc = GWL_ERR_CUDA;
    goto fail;
  }
  {
    std::vector<double> hf(P, 0.0);
    std::vector<float> hff(P, 0.0f);
    for (int64_t k = 0; k < N; ++k) {
      hf[k] = f[k];
      hff[k] = (float)f[k];
    }
    if ((rc = upload(a, &a->freq, hf))) goto fail;
    a->h_freq.assign(f, f + N);
    if (a->model == GWL_MODEL_SINEGAUSSIAN && (rc = upload(a, &a->freq_f, hff))) goto fail;
    if (a->model == GWL_MODEL_TAYLORF2) {
      // float-float phase basis: f^-5/3, f^-1, f^-2/3, f^-1/3, ln f, f^1/3, f^1/3 ln f, f^2/3
      std::vector<float2> basis((size_t)P * kNumBasis, make_float2(0.f, 0.f));
      for (int64_t k = 0; k < N; ++k) {
        const double x = f[k];
        if (!(x > 0)) continue;
        const double c3 = std::cbrt(x), lx = std::log(x);
        const double inv3 = 1.0 / c3;
        const double vals[kNumBasis] = {inv3 * inv3 * inv3 * inv3 * inv3, 1.0 / x, inv3 * inv3, inv3,
                                        lx, c3, c3 * lx, c3 * c3};
        for (int b = 0; b < kNumBasis; ++b) basis[(size_t)k * kNumBasis + b] = split_ff(vals[b]);
      }
      if ((rc = upload(a, &a->basis, basis))) goto fail;
      // float64 powers of f for the plain kernel
      std::vector<double4> ft((size_t)P, make_double4(0.0, 0.0, 0.0, 0.0));
      for (int64_t k = 0; k < N; ++k) {
        const double x = f[k];
        if (!(x > 0)) continue;
        ft[k] = make_double4(std::cbrt(x), std::log(x) / 3.0, std::pow(x, -5.0 / 3.0), std::pow(x, -7.0 / 6.0));
      }
      if ((rc = upload(a, &a->ftab, ft))) goto fail;
      // Taylor tables of the basis every kAnchorStep bins (f = k * df)
      a->n_anchors = N / kAnchorStep + 2;
      std::vector<float> anc((size_t)a->n_anchors * kAnchorFloats, 0.f);
      for (int64_t q = 1; q < a->n_anchors; ++q) {
        const double fa = (double)(q * kAnchorStep) * a->step;
        double T[kAnchorOrders][kNumBasis];
        basis_taylor(fa, a->step, T);
        float* dst = anc.data() + (size_t)q * kAnchorFloats;
        for (int n = 0; n < kAnchorOrders; ++n)
          for (int b = 0; b < kNumBasis; ++b) {
            const float2 v = split_ff(T[n][b]);
            dst[n * kNumBasis + b] = v.x;
            if (n < kAnchorFF) dst[kAnchorOrders * kNumBasis + n * kNumBasis + b] = v.y;
          }
      }
      if ((rc = upload(a, &a->anchors, anc))) goto fail;
      // float-float cos and sin of 2 pi q / kCosTable for the accurate kernel
      std::vector<float4> ct(kCosTable);
      for (int q = 0; q < kCosTable; ++q) {
        const double x = 2.0 * M_PI * q / kCosTable, c = std::cos(x), sn = std::sin(x);
        const float ch = (float)c, sh = (float)sn;
        ct[q] = make_float4(ch, (float)(c - (double)ch), sh, (float)(sn - (double)sh));
      }
      if ((rc = upload(a, &a->cos_tab, ct))) goto fail;
    }
    a->noise_lnl = 0.0;
    for (int d = 0; d < a->n_det; ++d) {
      const gwl_detector& det = desc->detectors[d];
      std::vector<double> s(2 * P, 0.0), ip(P, 0.0);
      KahanSum dd;
      for (int64_t k = 0; k < N; ++k) {
        if (!det.mask[k]) continue;
        s[2 * k] = det.strain[2 * k];
        s[2 * k + 1] = det.strain[2 * k + 1];
        const double S = det.psd[k];
        ip[k] = (std::isfinite(S) && S > 0) ? 1.0 / S : 0.0;
        // base.py:402-411: |<d|d>| / 2 with <a|b> = 4/T sum conj(a) b / S
        dd.add((s[2 * k] * s[2 * k] + s[2 * k + 1] * s[2 * k + 1]) * ip[k]);
      }
      a->noise_lnl -= std::fabs(4.0 / a->duration * dd.value() / 2.0);
      if ((rc = upload(a, &a->strain[d], s))) goto fail;
      if ((rc = upload(a, &a->inv_psd[d], ip))) goto fail;
      // mixed-precision weights, scaled into float32 range
      std::vector<double> wr(P, 0.0), wi(P, 0.0);
      double wmax = 0.0, vmax = 0.0;
      for (int64_t k = 0; k < N; ++k) {
        if (ip[k] == 0.0) continue;
        const double amp = a->model == GWL_MODEL_TAYLORF2 ? std::pow(f[k], -7.0 / 6.0) : 1.0;
        wr[k] = amp * s[2 * k] * ip[k];
        wi[k] = amp * s[2 * k + 1] * ip[k];
        wmax = std::max(wmax, std::max(std::fabs(wr[k]), std::fabs(wi[k])));
        vmax = std::max(vmax, ip[k]);
      }
      a->w_scale[d] = wmax > 0 ? wmax : 1.0;
      a->v_scale[d] = vmax > 0 ? vmax : 1.0;
      std::vector<float2> wf(P, make_float2(0.f, 0.f));
      std::vector<float> vf(P, 0.f);
      for (int64_t k = 0; k < N; ++k) {
        wf[k] = make_float2((float)(wr[k] / a->w_scale[d]), (float)(wi[k] / a->w_scale[d]));
        vf[k] = (float)(ip[k] / a->v_scale[d]);
      }
      if ((rc = upload(a, &a->w[d], wf))) goto fail;
      if (a->model == GWL_MODEL_TAYLORF2) {
        std::vector<uint2> wpol(P, make_uint2(0u, 0u));
        for (int64_t k = 0; k < N; ++k) {
          const double x = wr[k] / a->w_scale[d], y = wi[k] / a->w_scale[d];
          // odd bins carry -|w| at arg(w) + 1/2 cycle (the same term): a mean
          // error of the float32 cosine then cancels between neighbouring bins
          // instead of adding up coherently with the positive magnitudes
          const bool odd = (k & 1) != 0;
          const float mag = (float)(odd ? -std::hypot(x, y) : std::hypot(x, y));
          double cyc = std::atan2(y, x) / (2.0 * M_PI) + (odd ? 0.5 : 0.0);
          cyc -= std::floor(cyc);
          const uint32_t th = (uint32_t)(uint64_t)std::llround(cyc * 4294967296.0);  // 2^32 wraps to 0
          uint32_t mb;
          std::memcpy(&mb, &mag, 4);
          wpol[k] = make_uint2(mb, th);
        }
        if ((rc = upload(a, &a->wp[d], wpol))) goto fail;
        // the fast kernel's pairs: magnitudes side by side, then the angle at
        // the first bin of each 8-bin block and the increment over the
        // previous bin elsewhere (P is a multiple of 16)
        std::vector<uint4> wpair(P / 2);
        for (int64_t q = 0; q < P / 2; ++q) {
          const int64_t k = 2 * q;
          const uint32_t tau0 = (k % 8 == 0) ? wpol[k].y : wpol[k].y - wpol[k - 1].y;
          const uint32_t tau1 = wpol[k + 1].y - wpol[k].y;
          wpair[q] = make_uint4(wpol[k].x, wpol[k + 1].x, tau0, tau1);
        }
        if ((rc = upload(a, &a->wq[d], wpair))) goto fail;
      }
      if (a->model == GWL_MODEL_SINEGAUSSIAN) {
        // float-float inverse PSD for the float-float <h|h> of the mixed kernel
        std::vector<float> vl(P, 0.f);
        for (int64_t k = 0; k < N; ++k) vl[k] = (float)(ip[k] / a->v_scale[d] - (double)vf[k]);
        if ((rc = upload(a, &a->v[d], vf))) goto fail;
        if ((rc = upload(a, &a->v_lo[d], vl))) goto fail;
      } else {
        // <h|h> prefix sums of f^(-7/3) / S over the analysis grid
        std::vector<double> pre(N + 1, 0.0);
        KahanSum acc;
        for (int64_t k = 0; k < N; ++k) {
          if (ip[k] != 0.0 && f[k] > 0) acc.add(std::pow(f[k], -7.0 / 3.0) * ip[k]);
          pre[k + 1] = acc.value();
        }
        if ((rc = upload(a, &a->hh_prefix[d], pre))) goto fail;
        // refinement bound: prefix sums of the scaled weight magnitudes |w|^2,
        // and of |w| where the whitened data power 4 |d|^2 / (T S) exceeds
        // kRefineLoudPower (bins dominated by a signal, whose phase a template
        // can follow coherently)
        std::vector<double> p2(N + 1, 0.0), p1(N + 1, 0.0);
        KahanSum acc2, acc1;
        for (int64_t k = 0; k < N; ++k) {
          if (ip[k] != 0.0) {
            const double x = wr[k] / a->w_scale[d], y = wi[k] / a->w_scale[d];
            const double m2 = x * x + y * y;
            acc2.add(m2);
            const double pw = 4.0 / a->duration * (s[2 * k] * s[2 * k] + s[2 * k + 1] * s[2 * k + 1]) * ip[k];
            if (pw > kRefineLoudPower) acc1.add(std::sqrt(m2));
          }
          p2[k + 1] = acc2.value();
          p1[k + 1] = acc1.value();
        }
        if ((rc = upload(a, &a->rf_p2[d], p2))) goto fail;
        if ((rc = upload(a, &a->rf_p1[d], p1))) goto fail;
      }
    }
  }
  *out = a;
  return GWL_OK;
fail:
  for (void* p : a->tables) cudaFree(p);
  if (a->stream) cudaStreamDestroy(a->stream);
  side_stream_destroy(&a->side);
  delete a;
  return rc ? rc : GWL_ERR_CUDA;
}

int gwl_analysis_destroy(gwl_analysis* a) {
  if (!a) return GWL_OK;
  {
    std::lock_guard<std::mutex> g(a->mu);
    cudaStreamSynchronize(a->stream);
    free_workspace(a);
    if (a->blas) cublasDestroy(a->blas);
    for (void* p : a->tables) cudaFree(p);
    a->tables.clear();
    if (a->ev_begin) cudaEventDestroy(a->ev_begin);
    if (a->ev_end) cudaEventDestroy(a->ev_end);
    side_stream_destroy(&a->side);
    cudaStreamDestroy(a->stream);
  }
  delete a;
  return GWL_OK;
}

int gwl_analysis_resident_bytes(const gwl_analysis* a, size_t* bytes) {
  if (!a || !bytes) {
    set_error("null argument");
    return GWL_ERR_ARGUMENT;
  }
  *bytes = a->resident;
  return GWL_OK;
}

int gwl_set_profiling(gwl_analysis* a, int enable) {
  if (!a) {
    set_error("null argument");
    return GWL_ERR_ARGUMENT;
  }
  std::lock_guard<std::mutex> g(a->mu);
  if (enable && !a->ev_begin) {
    GWL_CUDA(cudaEventCreate(&a->ev_begin));
    GWL_CUDA(cudaEventCreate(&a->ev_end));
  }
  a->profiling = enable ? 1 : 0;
  a->ev_pending = 0;
  return GWL_OK;
}

int gwl_profile_last_kernel_ms(gwl_analysis* a, float* ms) {
  if (!a || !ms) {
    set_error("null argument");
    return GWL_ERR_ARGUMENT;
  }
  std::lock_guard<std::mutex> g(a->mu);
  if (!a->profiling || !a->ev_pending) {
    set_error("no profiled evaluation pending (enable gwl_set_profiling first)");
    return GWL_ERR_STATE;
  }
  GWL_CUDA(cudaEventSynchronize(a->ev_end));
  GWL_CUDA(cudaEventElapsedTime(ms, a->ev_begin, a->ev_end));
  a->ev_pending = 0;
  return GWL_OK;
}

int gwl_autotune(gwl_analysis* a, const double* params, int64_t B, void* stream, int32_t* chunks_per_group,
                 double* best_ms) {
  if (!a || !params || B <= 0) {
    set_error("gwl_autotune: null argument or empty batch");
    return GWL_ERR_ARGUMENT;
  }
  std::lock_guard<std::mutex> g(a->mu);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (a->model != GWL_MODEL_TAYLORF2 || a->time_marg || a->relbin || a->multiband || a->roq) {
    // nothing to tune: the other launch shapes are fixed
    if (chunks_per_group) *chunks_per_group = a->chunks_per_group;
    if (best_ms) *best_ms = 0.0;
    return GWL_OK;
  }
  cudaEvent_t e0, e1;
  GWL_CUDA(cudaEventCreate(&e0));
  GWL_CUDA(cudaEventCreate(&e1));
  const int candidates[] = {2, 3, 4, 6, 8, 12, 16};
  const int keep = a->chunks_per_group;
  int best = keep;
  float best_t = 0.f;
  int rc = GWL_OK;
  LaunchArgs L0 = make_args(a, B, GWL_PRECISION_MIXED);
  if ((rc = ensure_workspace(a, B, L0))) goto done;
  for (int c : candidates) {
    if (c > a->n_chunks_mixed && c != candidates[0]) break;
    a->chunks_per_group = c;
    // one untimed run, then the fastest of five timed runs of the whole launch
    // sequence (interference from other work only ever adds time)
    if ((rc = run_eval(a, params, B, GWL_PRECISION_MIXED, a->d_out, nullptr, nullptr, s))) goto done;
    float t[5];
    for (int r = 0; r < 5; ++r) {
      if (cudaEventRecord(e0, s) != cudaSuccess) { rc = GWL_ERR_CUDA; goto done; }
      if ((rc = run_eval(a, params, B, GWL_PRECISION_MIXED, a->d_out, nullptr, nullptr, s))) goto done;
      if (cudaEventRecord(e1, s) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
          cudaEventElapsedTime(&t[r], e0, e1) != cudaSuccess) {
        rc = GWL_ERR_CUDA;
        goto done;
      }
    }
    std::sort(t, t + 5);
    if (best_t == 0.f || t[0] < best_t) {
      best_t = t[0];
      best = c;
    }
  }
done:
  a->chunks_per_group = rc == GWL_OK ? best : keep;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc == GWL_OK) {
    if (chunks_per_group) *chunks_per_group = best;
    if (best_ms) *best_ms = best_t;
  }
  return rc;
}

int gwl_get_chunks_per_group(gwl_analysis* a, int32_t* chunks_per_group) {
  if (!a || !chunks_per_group) {
    set_error("null argument");
    return GWL_ERR_ARGUMENT;
  }
  *chunks_per_group = a->chunks_per_group;
  return GWL_OK;
}

int gwl_set_chunks_per_group(gwl_analysis* a, int32_t chunks_per_group) {
  if (!a || chunks_per_group < 1 || chunks_per_group > 1024) {
    set_error("chunks_per_group must be in [1, 1024]");
    return GWL_ERR_ARGUMENT;
  }
  std::lock_guard<std::mutex> g(a->mu);
  a->chunks_per_group = chunks_per_group;
  return GWL_OK;
}

int gwl_set_refinement(gwl_analysis* a, double tolerance) {
  if (!a || !std::isfinite(tolerance)) {
    set_error("refinement tolerance must be finite (<= 0 turns refinement off)");
    return GWL_ERR_ARGUMENT;
  }
  std::lock_guard<std::mutex> g(a->mu);
  a->refine_tol = tolerance;
  return GWL_OK;
}

int gwl_get_refinement(gwl_analysis* a, double* tolerance) {
  if (!a || !tolerance) {
    set_error("null argument");
    return GWL_ERR_ARGUMENT;
  }
  *tolerance = a->refine_tol;
  return GWL_OK;
}

int gwl_last_refined(gwl_analysis* a, void* stream, int64_t* count) {
  if (!a || !count) {
    set_error("null argument");
    return GWL_ERR_ARGUMENT;
  }
  *count = 0;
  std::lock_guard<std::mutex> g(a->mu);
  if (!a->last_rf_count) return GWL_OK;
  int n = 0;
  GWL_CUDA(cudaStreamSynchronize(static_cast<cudaStream_t>(stream)));
  GWL_CUDA(cudaMemcpy(&n, a->last_rf_count, sizeof(int), cudaMemcpyDeviceToHost));
  *count = n;
  return GWL_OK;
}

int gwl_noise_log_likelihood(gwl_analysis* a, double* out) {
  if (!a || !out) {
    set_error("null argument");
    return GWL_ERR_ARGUMENT;
  }
  *out = a->noise_lnl;
  return GWL_OK;
}

int gwl_set_time_marginalization(gwl_analysis* a, int enable, int jitter, double t_min, double t_max) {
  if (!a) {
    set_error("null argument");
    return GWL_ERR_ARGUMENT;
  }
  std::lock_guard<std::mutex> g(a->mu);
  if (enable) {
    if (!(t_max > t_min)) {
      set_error("time prior must have t_max > t_min");
      return GWL_ERR_ARGUMENT;
    }
    int m_odd = 0, log2n = 0;
    if (!fft_length_supported(a->n_bins - 1, &m_odd, &log2n)) {
      set_error("time marginalisation needs an FFT length n_bins - 1 = m 2^p with m odd, m <= " +
                std::to_string(kTmMaxOddFactor) + " and p >= 4");
      return GWL_ERR_UNSUPPORTED;
    }
  }
  a->time_marg = enable ? 1 : 0;
  a->jitter = jitter ? 1 : 0;
  a->t_min = t_min;
  a->t_max = t_max;
  return GWL_OK;
}

int gwl_set_time_prior(gwl_analysis* a, const double* density, int64_t n, double t0, double h) {
  if (!a || (n > 0 && !density)) {
    set_error("null argument");
    return GWL_ERR_ARGUMENT;
  }
  std::lock_guard<std::mutex> g(a->mu);
  if (n == 0) {  // back to the Uniform prior of the time-marginalisation window
    a->tm_prior = nullptr;
    a->tm_prior_f = nullptr;
    a->tm_prior_n = 0;
    return GWL_OK;
  }
  int e2 = 0;
  if (n < 4 || !(h > 0) || std::frexp(h, &e2) != 0.5 || !std::isfinite(t0) || std::fmod(t0, h) != 0.0) {
    set_error("time prior table: need n >= 4 nodes, h a power of two and t0 a multiple of h");
    return GWL_ERR_ARGUMENT;
  }
  std::vector<double> p(density, density + n);
  std::vector<float> pf(n);
  for (int64_t k = 0; k < n; ++k) {
    if (!(p[k] >= 0.0) || !std::isfinite(p[k])) {
      set_error("time prior table: densities must be finite and non-negative");
      return GWL_ERR_ARGUMENT;
    }
    pf[k] = (float)p[k];
  }
  // earlier tables stay allocated (in the analysis's table list) until the
  // analysis is destroyed: a launch in flight may still read them
  int rc;
  if ((rc = upload(a, &a->tm_prior, p))) return rc;
  if ((rc = upload(a, &a->tm_prior_f, pf))) return rc;
  a->tm_prior_n = n;
  a->tm_prior_t0 = t0;
  a->tm_prior_inv_h = 1.0 / h;
  return GWL_OK;
}

int gwl_set_phase_marginalization(gwl_analysis* a, int enable) {
  if (!a) {
    set_error("null argument");
    return GWL_ERR_ARGUMENT;
  }
  std::lock_guard<std::mutex> g(a->mu);
  a->phase_marg = enable ? 1 : 0;
  return GWL_OK;
}

int gwl_set_distance_slope(gwl_analysis* a, double max_slope) {
  if (!a) {
    set_error("null argument");
    return GWL_ERR_ARGUMENT;
  }
  if (!(max_slope >= 1.0) || !std::isfinite(max_slope)) {
    set_error("the distance slope bound d_ref / d_min must be finite and at least 1");
    return GWL_ERR_ARGUMENT;
  }
  std::lock_guard<std::mutex> g(a->mu);
  a->dist_slope = max_slope;
  return GWL_OK;
}

int gwl_set_distance_marginalization(gwl_analysis* a, int enable, const double* tx, int32_t nx, const double* ty,
                                     int32_t ny, const double* c, const double bbox[4], double reference_distance) {
  if (!a) {
    set_error("null argument");
    return GWL_ERR_ARGUMENT;
  }
  std::lock_guard<std::mutex> g(a->mu);
  if (!enable) {
    a->dist_marg = 0;
    return GWL_OK;
  }
  if (!tx || !ty || !c || !bbox || nx < 8 || ny < 8 || !(reference_distance > 0)) {
    set_error("distance spline needs knots (>= 8 per axis), coefficients, a box and a positive reference distance");
    return GWL_ERR_ARGUMENT;
  }
  std::vector<double> vx(tx, tx + nx), vy(ty, ty + ny), vc(c, c + (size_t)(nx - 4) * (ny - 4));
  int rc;
  if ((rc = upload(a, &a->tx, vx))) return rc;
  if ((rc = upload(a, &a->ty, vy))) return rc;
  if ((rc = upload(a, &a->tc, vc))) return rc;
  std::vector<float> fx(vx.begin(), vx.end()), fy(vy.begin(), vy.end()), fc(vc.begin(), vc.end());
  if ((rc = upload(a, &a->tx_f, fx))) return rc;
  if ((rc = upload(a, &a->ty_f, fy))) return rc;
  if ((rc = upload(a, &a->tc_f, fc))) return rc;
  a->nx = nx;
  a->ny = ny;
  for (int q = 0; q < 4; ++q) a->bbox[q] = bbox[q];
  a->ref_dist = reference_distance;
  a->dist_marg = 1;
  return GWL_OK;
}

int gwl_set_relative_binning(gwl_analysis* a, int enable, int32_t n_edges, const int64_t* edge_index,
                             const double* h0_inverse, const double* summary) {
  if (!a) {
    set_error("null argument");
    return GWL_ERR_ARGUMENT;
  }
  std::lock_guard<std::mutex> g(a->mu);
  if (!enable) {
    a->relbin = 0;
    return GWL_OK;
  }
  if (a->multiband || a->roq) {
    set_error("relative binning excludes multi-banding and ROQ");
    return GWL_ERR_UNSUPPORTED;
  }
  if (n_edges < 2 || !edge_index || !h0_inverse || !summary) {
    set_error("relative binning needs at least two bin edges, 1 / h0 at the edges and the summary data");
    return GWL_ERR_ARGUMENT;
  }
  std::vector<int64_t> idx(edge_index, edge_index + n_edges);
  std::vector<double> fe(n_edges);
  for (int32_t e = 0; e < n_edges; ++e) {
    if (idx[e] < 0 || idx[e] >= a->n_bins || (e > 0 && idx[e] <= idx[e - 1])) {
      set_error("bin edges must be increasing grid indices inside the frequency array");
      return GWL_ERR_ARGUMENT;
    }
    fe[e] = a->h_freq[idx[e]];
  }
  int rc;
  if ((rc = upload(a, &a->rb_index, idx))) return rc;
  if ((rc = upload(a, &a->rb_freq, fe))) return rc;
  const size_t nb = (size_t)(n_edges - 1);
  for (int d = 0; d < a->n_det; ++d) {
    std::vector<double2> h(n_edges);
    for (int32_t e = 0; e < n_edges; ++e)
      h[e] = make_double2(h0_inverse[((size_t)d * n_edges + e) * 2], h0_inverse[((size_t)d * n_edges + e) * 2 + 1]);
    std::vector<double> sm(summary + (size_t)d * nb * 6, summary + (size_t)(d + 1) * nb * 6);
    if ((rc = upload(a, &a->rb_h0inv[d], h))) return rc;
    if ((rc = upload(a, &a->rb_sum[d], sm))) return rc;
  }
  a->rb_edges = n_edges;
  a->h_rb_index = idx;
  a->rb_tm = 0;  // new bins need new time-marginalisation weights
  a->relbin = 1;
  return GWL_OK;
}

int gwl_set_relative_binning_time_weights(gwl_analysis* a, const double* weights) {
  if (!a || !weights) {
    set_error("null argument");
    return GWL_ERR_ARGUMENT;
  }
  std::lock_guard<std::mutex> g(a->mu);
  if (!a->relbin) {
    set_error("set the relative-binning bins first (gwl_set_relative_binning)");
    return GWL_ERR_ARGUMENT;
  }
  const std::vector<int64_t>& idx = a->h_rb_index;
  const int64_t k0 = idx.front(), k1 = idx.back();
  // bin b holds the grid indices [idx[b], idx[b + 1]); the last bin also idx.back()
  std::vector<int32_t> bin((size_t)(k1 - k0 + 1));
  for (size_t b = 0; b + 1 < idx.size(); ++b)
    for (int64_t k = idx[b]; k < idx[b + 1]; ++k) bin[(size_t)(k - k0)] = (int32_t)b;
  bin.back() = (int32_t)(idx.size() - 2);
  int rc;
  if ((rc = upload(a, &a->rb_bin, bin))) return rc;
  // mixed precision: f_k - (f_b + f_b+1) / 2 of each grid index, in float32
  std::vector<RbBinF> bx(bin.size());
  for (size_t q = 0; q < bin.size(); ++q) {
    const int32_t b = bin[q];
    const double fc = (a->h_freq[idx[(size_t)b]] + a->h_freq[idx[(size_t)b + 1]]) / 2;
    bx[q] = RbBinF{b, (float)(a->h_freq[(size_t)k0 + q] - fc)};
  }
  if ((rc = upload(a, &a->rb_bx, bx))) return rc;
  for (int d = 0; d < a->n_det; ++d) {
    std::vector<double2> w((size_t)a->n_bins);
    for (int64_t k = 0; k < a->n_bins; ++k)
      w[(size_t)k] = make_double2(weights[((size_t)d * a->n_bins + k) * 2], weights[((size_t)d * a->n_bins + k) * 2 + 1]);
    std::vector<float2> wf(bin.size());
    for (size_t q = 0; q < wf.size(); ++q)
      wf[q] = make_float2((float)w[(size_t)k0 + q].x, (float)w[(size_t)k0 + q].y);
    if ((rc = upload(a, &a->rb_g[d], w))) return rc;
    if ((rc = upload(a, &a->rb_gf[d], wf))) return rc;
  }
  a->rb_tm = 1;
  return GWL_OK;
}

int gwl_set_multiband(gwl_analysis* a, int enable, int64_t n_points, const double* frequencies,
                      const double* linear, const double* quadratic, int32_t n_bands, const int64_t* band_start,
                      const double* band_df) {
  if (!a) {
    set_error("null argument");
    return GWL_ERR_ARGUMENT;
  }
  std::lock_guard<std::mutex> g(a->mu);
  if (!enable) {
    a->multiband = 0;
    a->mb_fft = 0;
    return GWL_OK;
  }
  if (a->relbin || a->roq) {
    set_error("multi-banding excludes relative binning and ROQ");
    return GWL_ERR_UNSUPPORTED;
  }
  if (n_points < 1 || !frequencies || !linear || !quadratic || n_bands < 1 || !band_start || !band_df) {
    set_error("multi-banding needs the banded frequencies, both coefficient sets and the band layout");
    return GWL_ERR_ARGUMENT;
  }
  for (int32_t b = 0; b < n_bands; ++b) {
    if (band_start[b] < 0 || band_start[b + 1] < band_start[b] || band_start[b + 1] > n_points ||
        !(band_df[b] > 0)) {
      set_error("band layout must be increasing start indices within the banded frequencies, positive spacings");
      return GWL_ERR_ARGUMENT;
    }
    // the frequencies of a band must be uniform with its spacing (the kernel rotates from point to point)
    for (int64_t k = band_start[b] + 1; k < band_start[b + 1]; ++k) {
      const double step = frequencies[k] - frequencies[k - 1];
      if (std::fabs(step - band_df[b]) > 1e-9 * band_df[b]) {
        set_error("the frequencies of a band must be uniformly spaced by its spacing");
        return GWL_ERR_ARGUMENT;
      }
    }
  }
  std::vector<double> fr(frequencies, frequencies + n_points);
  std::vector<double4> pw(n_points, make_double4(0.0, 0.0, 0.0, 0.0));
  for (int64_t k = 0; k < n_points; ++k) {
    const double x = fr[k];
    if (!(x > 0) || !std::isfinite(x)) continue;
    pw[k] = make_double4(std::cbrt(x), std::log(x) / 3.0, std::pow(x, -5.0 / 3.0), std::pow(x, -7.0 / 6.0));
  }
  int rc;
  if ((rc = upload(a, &a->mb_freq, fr))) return rc;
  if ((rc = upload(a, &a->mb_pow, pw))) return rc;
  // mixed precision: float-float phase basis at the banded frequencies (the
  // functions of the analysis grid's basis table)
  std::vector<float2> mbb((size_t)n_points * kNumBasis, make_float2(0.f, 0.f));
  for (int64_t k = 0; k < n_points; ++k) {
    const double x = fr[k];
    if (!(x > 0) || !std::isfinite(x)) continue;
    const double c3 = std::cbrt(x), lx = std::log(x), inv3 = 1.0 / c3;
    const double vals[kNumBasis] = {inv3 * inv3 * inv3 * inv3 * inv3, 1.0 / x, inv3 * inv3, inv3, lx, c3, c3 * lx,
                                    c3 * c3};
    for (int b = 0; b < kNumBasis; ++b) mbb[(size_t)k * kNumBasis + b] = split_ff(vals[b]);
  }
  if ((rc = upload(a, &a->mb_basis, mbb))) return rc;
  for (int d = 0; d < a->n_det; ++d) {
    std::vector<double2> lin(n_points);
    for (int64_t k = 0; k < n_points; ++k)
      lin[k] = make_double2(linear[((size_t)d * n_points + k) * 2], linear[((size_t)d * n_points + k) * 2 + 1]);
    std::vector<double> quad(quadratic + (size_t)d * n_points, quadratic + (size_t)(d + 1) * n_points);
    if ((rc = upload(a, &a->mb_lin[d], lin))) return rc;
    if ((rc = upload(a, &a->mb_quad[d], quad))) return rc;
    // mixed precision: L f^(-7/6) scaled into float32 range, and prefix sums of f^(-7/3) quad
    std::vector<double> lr(n_points, 0.0), li(n_points, 0.0), qp(n_points + 1, 0.0);
    double lmax = 0.0;
    KahanSum acc;
    for (int64_t k = 0; k < n_points; ++k) {
      const double x = fr[k];
      if (x > 0 && std::isfinite(x)) {
        const double a76 = std::pow(x, -7.0 / 6.0);
        lr[k] = lin[k].x * a76;
        li[k] = lin[k].y * a76;
        lmax = std::max(lmax, std::max(std::fabs(lr[k]), std::fabs(li[k])));
        acc.add(a76 * a76 * quad[k]);
      }
      qp[k + 1] = acc.value();
    }
    a->mb_lw_scale[d] = lmax > 0 ? lmax : 1.0;
    std::vector<float2> lw(n_points);
    std::vector<double> l2(n_points + 1, 0.0);
    KahanSum acc2;
    for (int64_t k = 0; k < n_points; ++k) {
      lw[k] = make_float2((float)(lr[k] / a->mb_lw_scale[d]), (float)(li[k] / a->mb_lw_scale[d]));
      acc2.add((double)lw[k].x * lw[k].x + (double)lw[k].y * lw[k].y);
      l2[k + 1] = acc2.value();
    }
    if ((rc = upload(a, &a->mb_lw[d], lw))) return rc;
    if ((rc = upload(a, &a->mb_qprefix[d], qp))) return rc;
    if ((rc = upload(a, &a->mb_l2prefix[d], l2))) return rc;
  }
  std::vector<int64_t> bs(band_start, band_start + n_bands + 1);
  std::vector<double> bd(band_df, band_df + n_bands);
  if ((rc = upload(a, &a->mb_band_start, bs))) return rc;
  a->mb_band_start_h = bs;
  a->mb_freq_h = fr;
  a->mb_fft = 0;  // new bands need new IFFT-FFT tables
  if ((rc = upload(a, &a->mb_band_df, bd))) return rc;
  a->mb_bands = n_bands;
  a->mb_points = n_points;
  a->mb_tm = 0;  // new bands need new time-marginalisation tables
  a->multiband = 1;
  return GWL_OK;
}

int gwl_set_multiband_ifft_fft(gwl_analysis* a, int enable, const int32_t* ks, const int32_t* m,
                               const double* scale, const double* sqrt_window, const double* odd_weights) {
  if (!a) {
    set_error("null argument");
    return GWL_ERR_ARGUMENT;
  }
  std::lock_guard<std::mutex> g(a->mu);
  if (!enable) {
    a->mb_fft = 0;
    return GWL_OK;
  }
  if (!a->multiband) {
    set_error("set the bands first (gwl_set_multiband)");
    return GWL_ERR_ARGUMENT;
  }
  if (!ks || !m || !scale || !sqrt_window || !odd_weights) {
    set_error("the IFFT-FFT <h|h> needs K_s, M, the scales, the window roots and the odd-bin weights of every band");
    return GWL_ERR_ARGUMENT;
  }
  const int nb = a->mb_bands;
  if (m[0] != 0) {
    set_error("band 0's <h|h> is in the quadratic coefficients: m[0] must be 0");
    return GWL_ERR_ARGUMENT;
  }
  int64_t total = 0;
  int log2m_max = 2;
  for (int b = 1; b < nb; ++b) {
    const int64_t M = m[b], nk = a->mb_band_start_h[b + 1] - a->mb_band_start_h[b];
    if (M < 4 || M > ((int64_t)1 << 22) || (M & (M - 1)) != 0) {
      set_error("each band's M must be a power of two between 4 and 2^22");
      return GWL_ERR_ARGUMENT;
    }
    // the band's bins m = K_s .. K_s + n - 1 and their mirrors M - m must be
    // distinct and exclude 0 and M / 2
    if (nk > 0 && (ks[b] < 1 || (int64_t)ks[b] + nk - 1 >= M / 2)) {
      set_error("each band's bins must satisfy 1 <= K_s and K_s + n_points - 1 < M / 2");
      return GWL_ERR_ARGUMENT;
    }
    if (!(scale[b] >= 0) || !std::isfinite(scale[b])) {
      set_error("the band scales 4 / That must be finite and non-negative");
      return GWL_ERR_ARGUMENT;
    }
    int l = 0;
    while ((int64_t)1 << l < M) ++l;
    log2m_max = std::max(log2m_max, l);
    total += M / 2;
  }
  int rc;
  std::vector<double> sw(sqrt_window, sqrt_window + a->mb_points);
  for (double v : sw) {
    if (!std::isfinite(v)) {
      set_error("the window roots must be finite");
      return GWL_ERR_ARGUMENT;
    }
  }
  if ((rc = upload(a, &a->mbf_sqrtw, sw))) return rc;
  for (int d = 0; d < a->n_det; ++d) {
    std::vector<double> od(odd_weights + (size_t)d * total, odd_weights + (size_t)(d + 1) * total);
    if ((rc = upload(a, &a->mbf_odd[d], od))) return rc;
  }
  // mixed precision: the odd-bin weights as float-float pairs over each band's largest
  std::vector<double> odd_scale((size_t)nb, 1.0);
  {
    int64_t off0 = 0;
    for (int b = 1; b < nb; ++b) {
      double mx = 0.0;
      for (int d = 0; d < a->n_det; ++d)
        for (int64_t j = 0; j < m[b] / 2; ++j) mx = std::max(mx, std::fabs(odd_weights[(size_t)d * total + off0 + j]));
      odd_scale[(size_t)b] = mx > 0 ? mx : 1.0;
      off0 += m[b] / 2;
    }
    for (int d = 0; d < a->n_det; ++d) {
      std::vector<float2> o32((size_t)total);
      int64_t off1 = 0;
      for (int b = 1; b < nb; ++b) {
        for (int64_t j = 0; j < m[b] / 2; ++j)
          o32[(size_t)(off1 + j)] = split_ff(odd_weights[(size_t)d * total + off1 + j] / odd_scale[(size_t)b]);
        off1 += m[b] / 2;
      }
      if ((rc = upload(a, &a->mbf_odd32[d], o32))) return rc;
    }
  }
  // exp(-i pi k / 2^log2m_max), k < 2^(log2m_max + 1): the whole circle, as
  // the radix-4 passes read up to 3/2 of the half circle
  const int64_t n_tw = (int64_t)1 << log2m_max;
  std::vector<double2> tw((size_t)(2 * n_tw));
  for (int64_t k = 0; k < 2 * n_tw; ++k) {
    const double th = M_PI * (double)k / (double)n_tw;
    tw[(size_t)k] = make_double2(std::cos(th), -std::sin(th));
  }
  if ((rc = upload(a, &a->mbf_tw, tw))) return rc;
  std::vector<float2> tw32(tw.size());
  for (size_t k = 0; k < tw.size(); ++k) tw32[k] = make_float2((float)tw[k].x, (float)tw[k].y);
  if ((rc = upload(a, &a->mbf_tw32, tw32))) return rc;
  // mixed precision: sqrt(w_k) f_k^(-7/6), scaled to at most one
  std::vector<double> awd(sw.size(), 0.0);
  double aw_max = 0.0;
  for (size_t k = 0; k < sw.size(); ++k) {
    const double f = k < a->mb_freq_h.size() ? a->mb_freq_h[k] : 0.0;
    if (f > 0 && std::isfinite(f)) awd[k] = sw[k] * std::pow(f, -7.0 / 6.0);
    aw_max = std::max(aw_max, std::fabs(awd[k]));
  }
  a->mbf_aw_scale = aw_max > 0 ? aw_max : 1.0;
  std::vector<float> aw(sw.size());
  for (size_t k = 0; k < sw.size(); ++k) aw[k] = (float)(awd[k] / a->mbf_aw_scale);
  if ((rc = upload(a, &a->mbf_aw, aw))) return rc;
  a->mbf_log2m_max = log2m_max;
  a->mbf_bands.clear();
  int64_t off = 0;
  for (int b = 1; b < nb; ++b) {
    MbFftBand bd;
    std::memset(&bd, 0, sizeof(bd));
    bd.band = b;
    bd.ks = ks[b];
    int l = 0;
    while (((int64_t)1 << l) < m[b]) ++l;
    bd.log2m = l;
    bd.log2m_max = log2m_max;
    bd.in_smem = mb_hh_fft_smem(l) > 0;
    bd.scale = scale[b];
    for (int d = 0; d < a->n_det; ++d) {
      bd.odd[d] = a->mbf_odd[d] + off;
      bd.odd32[d] = a->mbf_odd32[d] + off;
    }
    bd.odd32_scale = odd_scale[(size_t)b];
    bd.sqrtw = a->mbf_sqrtw;
    bd.tw = a->mbf_tw;
    bd.tw32 = a->mbf_tw32;
    bd.aw = a->mbf_aw;
    bd.aw_scale = a->mbf_aw_scale;
    a->mbf_bands.push_back(bd);
    off += m[b] / 2;
  }
  a->mb_fft = nb > 1;
  return GWL_OK;
}

int gwl_set_multiband_time_marginalization(gwl_analysis* a, int64_t n_fft, const int32_t* index_start,
                                           const int32_t* source, double delta_tc, double antenna_time) {
  if (!a || !index_start || !source) {
    set_error("null argument");
    return GWL_ERR_ARGUMENT;
  }
  std::lock_guard<std::mutex> g(a->mu);
  if (!a->multiband) {
    set_error("set the bands first (gwl_set_multiband)");
    return GWL_ERR_ARGUMENT;
  }
  if (n_fft < 2 || (n_fft & (n_fft - 1)) != 0 || n_fft > ((int64_t)1 << 26)) {
    set_error("the multi-banding FFT length must be a power of two");
    return GWL_ERR_ARGUMENT;
  }
  if (!(delta_tc > 0) || !std::isfinite(antenna_time)) {
    set_error("delta_tc must be positive and the antenna time finite");
    return GWL_ERR_ARGUMENT;
  }
  std::vector<int32_t> ptr(index_start, index_start + n_fft + 1);
  if (ptr[0] != 0 || ptr[(size_t)n_fft] != (int32_t)a->mb_points) {
    set_error("index_start must run from 0 to the number of banded points");
    return GWL_ERR_ARGUMENT;
  }
  for (int64_t k = 0; k < n_fft; ++k)
    if (ptr[(size_t)k + 1] < ptr[(size_t)k]) {
      set_error("index_start must be non-decreasing");
      return GWL_ERR_ARGUMENT;
    }
  std::vector<int32_t> src(source, source + a->mb_points);
  std::vector<char> seen((size_t)a->mb_points, 0);
  for (int32_t c : src) {
    const int64_t j = c >= 0 ? c : -(int64_t)c - 1;
    if (j >= a->mb_points || seen[(size_t)j]) {
      set_error("source must list every banded point exactly once");
      return GWL_ERR_ARGUMENT;
    }
    seen[(size_t)j] = 1;
  }
  int rc;
  if ((rc = upload(a, &a->mb_tm_ptr, ptr))) return rc;
  if ((rc = upload(a, &a->mb_tm_src, src))) return rc;
  a->mb_tm_n = n_fft;
  a->mb_tm_delta_tc = delta_tc;
  a->mb_tm_antenna_time = antenna_time;
  a->mb_tm = 1;
  return GWL_OK;
}

namespace {
std::vector<double4> node_powers(const std::vector<double>& f) {
  std::vector<double4> pw(f.size(), make_double4(0.0, 0.0, 0.0, 0.0));
  for (size_t k = 0; k < f.size(); ++k) {
    const double x = f[k];
    if (!(x > 0) || !std::isfinite(x)) continue;
    pw[k] = make_double4(std::cbrt(x), std::log(x) / 3.0, std::pow(x, -5.0 / 3.0), std::pow(x, -7.0 / 6.0));
  }
  return pw;
}
}  // namespace

int gwl_set_roq(gwl_analysis* a, int enable, int32_t n_linear, const double* nodes_linear, int32_t n_quadratic,
                const double* nodes_quadratic, int64_t n_time, int64_t time_start_index, double time_step,
                const double* linear_weights, const double* quadratic_weights) {
  if (!a) {
    set_error("null argument");
    return GWL_ERR_ARGUMENT;
  }
  std::lock_guard<std::mutex> g(a->mu);
  if (!enable) {
    a->roq = 0;
    return GWL_OK;
  }
  if (a->relbin || a->multiband) {
    set_error("ROQ excludes relative binning and multi-banding");
    return GWL_ERR_UNSUPPORTED;
  }
  if (n_linear < 1 || n_quadratic < 1 || n_time < 5 || !(time_step > 0) || time_start_index < 0 || !nodes_linear ||
      !nodes_quadratic || !linear_weights || !quadratic_weights) {
    set_error("ROQ needs nodes, at least five time samples with a positive step and both weight sets");
    return GWL_ERR_ARGUMENT;
  }
  std::vector<double> fl(nodes_linear, nodes_linear + n_linear), fq(nodes_quadratic, nodes_quadratic + n_quadratic);
  int rc;
  if ((rc = upload(a, &a->roq_fl, fl))) return rc;
  if ((rc = upload(a, &a->roq_fq, fq))) return rc;
  if ((rc = upload(a, &a->roq_pl, node_powers(fl)))) return rc;
  if ((rc = upload(a, &a->roq_pq, node_powers(fq)))) return rc;
  const size_t per = (size_t)n_time * n_linear;
  for (int d = 0; d < a->n_det; ++d) {
    std::vector<double2> wl(per);
    for (size_t k = 0; k < per; ++k)
      wl[k] = make_double2(linear_weights[((size_t)d * per + k) * 2], linear_weights[((size_t)d * per + k) * 2 + 1]);
    std::vector<double> wq(quadratic_weights + (size_t)d * n_quadratic,
                           quadratic_weights + (size_t)(d + 1) * n_quadratic);
    if ((rc = upload(a, &a->roq_wl[d], wl))) return rc;
    if ((rc = upload(a, &a->roq_wq[d], wq))) return rc;
    // float32 copy with the nodes zero-padded to kRoqSplits groups of ks, and
    // per group the largest row norm, for the mixed time marginalisation
    const int ks = (n_linear + kRoqSplits - 1) / kRoqSplits, np = ks * kRoqSplits;
    std::vector<float2> w32((size_t)n_time * np, make_float2(0.f, 0.f));
    double wmax[kRoqSplits] = {};
    for (int64_t k = 0; k < n_time; ++k) {
      double n2[kRoqSplits] = {};
      for (int q = 0; q < n_linear; ++q) {
        const double2 v = wl[(size_t)k * n_linear + q];
        w32[(size_t)k * np + q] = make_float2((float)v.x, (float)v.y);
        n2[q / ks] += v.x * v.x + v.y * v.y;
      }
      for (int sp = 0; sp < kRoqSplits; ++sp) wmax[sp] = std::max(wmax[sp], std::sqrt(n2[sp]));
    }
    if ((rc = upload(a, &a->roq_wl32[d], w32))) return rc;
    for (int sp = 0; sp < kRoqSplits; ++sp) a->roq_wnorm[d][sp] = (float)wmax[sp];
    a->roq_ks = ks;
    a->roq_nl_pad = np;
  }
  a->roq_nl = n_linear;
  a->roq_nq = n_quadratic;
  a->roq_n_time = n_time;
  a->roq_time_start = time_start_index;
  a->roq_dt = time_step;
  a->roq_tm = 0;  // new weights need a new time-marginalisation grid
  a->roq = 1;
  return GWL_OK;
}

int gwl_set_roq_time_marginalization(gwl_analysis* a, int64_t n_times, const double* times, double delta_tc,
                                     double antenna_time) {
  if (!a || !times) {
    set_error("null argument");
    return GWL_ERR_ARGUMENT;
  }
  std::lock_guard<std::mutex> g(a->mu);
  if (!a->roq) {
    set_error("set the ROQ weights first (gwl_set_roq)");
    return GWL_ERR_ARGUMENT;
  }
  if (n_times < 1 || !(delta_tc > 0) || !std::isfinite(antenna_time)) {
    set_error("ROQ time marginalisation needs at least one time, a positive delta_tc and a finite antenna time");
    return GWL_ERR_ARGUMENT;
  }
  std::vector<double> t(times, times + n_times);
  for (int64_t j = 1; j < n_times; ++j)
    if (!(t[(size_t)j] > t[(size_t)j - 1])) {
      set_error("ROQ marginalisation times must increase");
      return GWL_ERR_ARGUMENT;
    }
  // rows one chunk of samples reads per detector: the span of its detector
  // times on the weight grid plus the five-sample stencil (the jitter shifts
  // both ends alike); chunks of 1024 samples, halved until they fit
  const double t0 = (double)a->roq_time_start * a->roq_dt;
  const double space = (double)(a->roq_time_start + 1) * a->roq_dt - t0;
  int64_t chunk = 1024, rows = 0;
  for (;; chunk /= 2) {
    double span = 0.0;
    for (int64_t j0 = 0; j0 < n_times; j0 += chunk)
      span = std::max(span, t[(size_t)std::min(n_times, j0 + chunk) - 1] - t[(size_t)j0]);
    rows = (int64_t)std::ceil(span / space) + 8;
    const size_t smem = (size_t)a->n_det * ((size_t)a->roq_nl + (size_t)rows) * sizeof(double2);
    if (smem <= 200 * 1024) break;
    if (chunk == 1) {
      set_error("ROQ time marginalisation: " + std::to_string(a->roq_nl) +
                " linear nodes per detector exceed the shared memory of one CTA");
      return GWL_ERR_UNSUPPORTED;
    }
  }
  int rc;
  if ((rc = upload(a, &a->roq_tm_times, t))) return rc;
  // the mixed kernel's weight-grid index of each sample, (t_j - start_0 - t0) / dt
  // in float64 split into its floor and a float32 fraction (per point and
  // detector it adds ((start_0 - start_d) + delay_d + jitter) / dt, split alike)
  std::vector<int2> gidx((size_t)n_times);
  for (int64_t j = 0; j < n_times; ++j) {
    const double x = ((t[(size_t)j] - a->geom[0].start_time) - t0) / space;
    const double fx = std::floor(x);
    const float fr = (float)(x - fx);
    int bits;
    std::memcpy(&bits, &fr, 4);
    gidx[(size_t)j] = make_int2((int)fx, bits);
  }
  if ((rc = upload(a, &a->roq_tm_g, gidx))) return rc;
  a->roq_tm_n = n_times;
  a->roq_tm_chunk = chunk;
  a->roq_tm_rows = rows;
  a->roq_tm_delta_tc = delta_tc;
  a->roq_tm_antenna_time = antenna_time;
  a->roq_tm = 1;
  return GWL_OK;
}

int gwl_trace_push(const char* name) {
  nvtxRangePushA(name ? name : "gwl");
  return GWL_OK;
}

int gwl_trace_pop(void) {
  nvtxRangePop();
  return GWL_OK;
}

int gwl_eval_device(gwl_analysis* a, const double* params, int64_t B, int32_t precision, double* out, void* stream) {
  if (!a || (B > 0 && (!params || !out))) {
    set_error("null argument");
    return GWL_ERR_ARGUMENT;
  }
  std::lock_guard<std::mutex> g(a->mu);
  TraceRange tr("gwl_eval_device");
  return run_eval(a, params, B, precision, out, nullptr, nullptr, static_cast<cudaStream_t>(stream));
}

int gwl_inner_products_device(gwl_analysis* a, const double* params, int64_t B, int32_t precision, double* d_inner_h,
                              double* h_inner_h, void* stream) {
  if (!a || (B > 0 && (!params || !d_inner_h || !h_inner_h))) {
    set_error("null argument");
    return GWL_ERR_ARGUMENT;
  }
  std::lock_guard<std::mutex> g(a->mu);
  const int saved = a->time_marg;
  a->time_marg = 0;
  const int rc = run_eval(a, params, B, precision, nullptr, d_inner_h, h_inner_h, static_cast<cudaStream_t>(stream));
  a->time_marg = saved;
  return rc;
}

int gwl_time_series_device(gwl_analysis* a, const double* params, int64_t B, double* series, double* h_inner_h,
                           void* stream) {
  if (!a || (B > 0 && (!params || !series || !h_inner_h))) {
    set_error("null argument");
    return GWL_ERR_ARGUMENT;
  }
  std::lock_guard<std::mutex> g(a->mu);
  if (!a->time_marg) {
    set_error("gwl_time_series_device needs time marginalisation enabled");
    return GWL_ERR_ARGUMENT;
  }
  if (a->roq && !a->roq_tm) {
    set_error("gwl_time_series_device needs the ROQ time-marginalisation grid (gwl_set_roq_time_marginalization)");
    return GWL_ERR_ARGUMENT;
  }
  if (B <= 0) return GWL_OK;
  LaunchArgs L = make_args(a, B, GWL_PRECISION_FP64);
  int rc = ensure_workspace(a, B, L);
  if (rc) return rc;
  // the marginalised lnL goes to the work space's result slots
  return run_eval(a, params, B, GWL_PRECISION_FP64, a->d_out, nullptr, h_inner_h, static_cast<cudaStream_t>(stream),
                  series);
}

namespace {
// One evaluation of the B points in the pinned staging buffer h_params into
// h_out (the caller holds the analysis lock): upload, launch sequence,
// download of the results and the device status word, one synchronisation.
int eval_staged(gwl_analysis* a, int64_t B, int32_t precision) {
  TraceRange tr("gwl_eval_host");
  {
    TraceRange t1("h2d");
    GWL_CUDA(cudaMemcpyAsync(a->d_params, a->h_params, sizeof(double) * GWL_NPARAM * B, cudaMemcpyHostToDevice,
                             a->stream));
  }
  {
    TraceRange t2("launch");
    int rc = run_eval(a, a->d_params, B, precision, a->d_out, nullptr, nullptr, a->stream);
    if (rc) return rc;
  }
  int* h_status = reinterpret_cast<int*>(a->h_out + B);
  {
    TraceRange t3("readback");
    GWL_CUDA(cudaMemcpyAsync(a->h_out, a->d_out, sizeof(double) * B, cudaMemcpyDeviceToHost, a->stream));
    GWL_CUDA(cudaMemcpyAsync(h_status, a->d_status, sizeof(int), cudaMemcpyDeviceToHost, a->stream));
    GWL_CUDA(cudaStreamSynchronize(a->stream));
  }
  if (*h_status != kDevStatusOk) {
    const int code = *h_status;
    cudaMemset(a->d_status, 0, sizeof(int));
    if (code == kDevStatusIndex) {
      set_error("an index check of the checked build failed (the access was skipped)");
      return GWL_ERR_CHECK;
    }
    set_error("a bounded device wait gave up (bulk copy did not complete)");
    return GWL_ERR_TIMEOUT;
  }
  return GWL_OK;
}
}  // namespace

int gwl_eval_host(gwl_analysis* a, const double* params, int64_t B, int32_t precision, double* out) {
  if (!a || (B > 0 && (!params || !out))) {
    set_error("null argument");
    return GWL_ERR_ARGUMENT;
  }
  if (B <= 0) return GWL_OK;
  std::lock_guard<std::mutex> g(a->mu);
  LaunchArgs L = make_args(a, B, precision);
  int rc = ensure_workspace(a, B, L);
  if (rc) return rc;
  // stage through pinned buffers so that both copies are true async DMA
  std::memcpy(a->h_params, params, sizeof(double) * GWL_NPARAM * B);
  if ((rc = eval_staged(a, B, precision))) return rc;
  std::memcpy(out, a->h_out, sizeof(double) * B);
  return GWL_OK;
}

int gwl_host_buffers(gwl_analysis* a, int64_t B, double** params, double** out) {
  if (!a || B <= 0 || !params || !out) {
    set_error("null argument or empty batch");
    return GWL_ERR_ARGUMENT;
  }
  std::lock_guard<std::mutex> g(a->mu);
  LaunchArgs L = make_args(a, B, GWL_PRECISION_FP64);
  int rc = ensure_workspace(a, B, L);
  if (rc) return rc;
  *params = a->h_params;
  *out = a->h_out;
  return GWL_OK;
}

int gwl_eval_host_staged(gwl_analysis* a, int64_t B, int32_t precision) {
  if (!a || B < 0) {
    set_error("null argument or negative batch size");
    return GWL_ERR_ARGUMENT;
  }
  if (B == 0) return GWL_OK;
  std::lock_guard<std::mutex> g(a->mu);
  if (B > a->ws_B || !a->h_params) {
    set_error("gwl_eval_host_staged: call gwl_host_buffers for this batch size first");
    return GWL_ERR_ARGUMENT;
  }
  LaunchArgs L = make_args(a, B, precision);
  int rc = ensure_workspace(a, B, L);  // the time-marginalisation work space may still be missing
  if (rc) return rc;
  return eval_staged(a, B, precision);
}

int gwl_source_polarizations(int32_t model, const double* frequency, int64_t n, const double* params,
                             double minimum_frequency, double* plus, double* cross) {
  if (!frequency || !params || !plus || !cross || n <= 0) {
    set_error("null argument or empty grid");
    return GWL_ERR_ARGUMENT;
  }
  if (model != GWL_MODEL_SINEGAUSSIAN && model != GWL_MODEL_TAYLORF2) {
    set_error("unsupported source model");
    return GWL_ERR_UNSUPPORTED;
  }
  double *df = nullptr, *dp = nullptr, *dplus = nullptr, *dcross = nullptr;
  int rc = GWL_OK;
  cudaError_t e;
  if ((e = cudaMalloc(&df, n * sizeof(double))) != cudaSuccess) goto cuda_fail;
  if ((e = cudaMalloc(&dp, GWL_NPARAM * sizeof(double))) != cudaSuccess) goto cuda_fail;
  if ((e = cudaMalloc(&dplus, 2 * n * sizeof(double))) != cudaSuccess) goto cuda_fail;
  if ((e = cudaMalloc(&dcross, 2 * n * sizeof(double))) != cudaSuccess) goto cuda_fail;
  if ((e = cudaMemcpy(df, frequency, n * sizeof(double), cudaMemcpyHostToDevice)) != cudaSuccess) goto cuda_fail;
  if ((e = cudaMemcpy(dp, params, GWL_NPARAM * sizeof(double), cudaMemcpyHostToDevice)) != cudaSuccess) goto cuda_fail;
  if ((e = launch_source_polarizations(model, df, n, dp, minimum_frequency, dplus, dcross, 0)) != cudaSuccess)
    goto cuda_fail;
  if ((e = cudaMemcpy(plus, dplus, 2 * n * sizeof(double), cudaMemcpyDeviceToHost)) != cudaSuccess) goto cuda_fail;
  if ((e = cudaMemcpy(cross, dcross, 2 * n * sizeof(double), cudaMemcpyDeviceToHost)) != cudaSuccess) goto cuda_fail;
  goto done;
cuda_fail:
  set_error(std::string("source polarisations: ") + cudaGetErrorString(e));
  rc = GWL_ERR_CUDA;
done:
  cudaFree(df);
  cudaFree(dp);
  cudaFree(dplus);
  cudaFree(dcross);
  return rc;
}

int gwl_detector_response(const gwl_detector* det, const double* frequency, int64_t n, const double* plus,
                          const double* cross, const double* params, double* response) {
  if (!det || !frequency || !plus || !cross || !params || !response || n <= 0 || !det->mask) {
    set_error("null argument or empty grid");
    return GWL_ERR_ARGUMENT;
  }
  DetGeom g;
  std::memcpy(g.vertex, det->vertex, sizeof(g.vertex));
  std::memcpy(g.tensor, det->tensor, sizeof(g.tensor));
  g.start_time = det->start_time;
  std::vector<double> masked_plus(2 * n), masked_cross(2 * n);
  for (int64_t k = 0; k < n; ++k) {
    const double m = det->mask[k] ? 1.0 : 0.0;
    masked_plus[2 * k] = plus[2 * k] * m;
    masked_plus[2 * k + 1] = plus[2 * k + 1] * m;
    masked_cross[2 * k] = cross[2 * k] * m;
    masked_cross[2 * k + 1] = cross[2 * k + 1] * m;
  }
  double *df = nullptr, *dp = nullptr, *dplus = nullptr, *dcross = nullptr, *dr = nullptr;
  int rc = GWL_OK;
  cudaError_t e;
  if ((e = cudaMalloc(&df, n * sizeof(double))) != cudaSuccess) goto cuda_fail;
  if ((e = cudaMalloc(&dp, GWL_NPARAM * sizeof(double))) != cudaSuccess) goto cuda_fail;
  if ((e = cudaMalloc(&dplus, 2 * n * sizeof(double))) != cudaSuccess) goto cuda_fail;
  if ((e = cudaMalloc(&dcross, 2 * n * sizeof(double))) != cudaSuccess) goto cuda_fail;
  if ((e = cudaMalloc(&dr, 2 * n * sizeof(double))) != cudaSuccess) goto cuda_fail;
  if ((e = cudaMemcpy(df, frequency, n * sizeof(double), cudaMemcpyHostToDevice)) != cudaSuccess) goto cuda_fail;
  if ((e = cudaMemcpy(dp, params, GWL_NPARAM * sizeof(double), cudaMemcpyHostToDevice)) != cudaSuccess) goto cuda_fail;
  if ((e = cudaMemcpy(dplus, masked_plus.data(), 2 * n * sizeof(double), cudaMemcpyHostToDevice)) != cudaSuccess)
    goto cuda_fail;
  if ((e = cudaMemcpy(dcross, masked_cross.data(), 2 * n * sizeof(double), cudaMemcpyHostToDevice)) != cudaSuccess)
    goto cuda_fail;
  if ((e = launch_detector_response(g, df, n, dplus, dcross, dp, dr, 0)) != cudaSuccess) goto cuda_fail;
  if ((e = cudaMemcpy(response, dr, 2 * n * sizeof(double), cudaMemcpyDeviceToHost)) != cudaSuccess) goto cuda_fail;
  goto done;
cuda_fail:
  set_error(std::string("detector response: ") + cudaGetErrorString(e));
  rc = GWL_ERR_CUDA;
done:
  cudaFree(df);
  cudaFree(dp);
  cudaFree(dplus);
  cudaFree(dcross);
  cudaFree(dr);
  return rc;
}

int gwl_batcher_create(gwl_batcher** out) {
  if (!out) {
    set_error("null argument");
    return GWL_ERR_ARGUMENT;
  }
  auto* b = new gwl_batcher();
  cudaError_t e = cudaMalloc(&b->d_counter, kMultiCounters * sizeof(int));
  if (e == cudaSuccess) e = cudaMalloc(&b->d_status, sizeof(int));
  if (e == cudaSuccess) e = cudaMemset(b->d_status, 0, sizeof(int));
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->staged, cudaEventDisableTiming);
  if (e == cudaSuccess) e = side_stream_create(&b->side);
  if (e != cudaSuccess) {
    set_error(std::string("gwl_batcher_create: ") + cudaGetErrorString(e));
    cudaFree(b->d_counter);
    cudaFree(b->d_status);
    side_stream_destroy(&b->side);
    delete b;
    return GWL_ERR_CUDA;
  }
  *out = b;
  return GWL_OK;
}

int gwl_batcher_destroy(gwl_batcher* b) {
  if (!b) return GWL_OK;
  {
    std::lock_guard<std::mutex> g(b->mu);
    cudaDeviceSynchronize();
    drop_graphs(b);
    cudaFree(b->d_args);
    cudaFreeHost(b->h_args);
    cudaFree(b->d_off);
    cudaFreeHost(b->h_off);
    cudaFree(b->d_units);
    cudaFreeHost(b->h_units);
    cudaFree(b->d_counter);
    cudaFree(b->d_rec);
    cudaFree(b->d_part);
    cudaFree(b->d_order);
    cudaFree(b->d_hist);
    cudaFree(b->d_status);
    cudaEventDestroy(b->staged);
    side_stream_destroy(&b->side);
  }
  delete b;
  return GWL_OK;
}

int gwl_batcher_use_graphs(gwl_batcher* b, int enable) {
  if (!b) {
    set_error("null argument");
    return GWL_ERR_ARGUMENT;
  }
  std::lock_guard<std::mutex> g(b->mu);
  b->use_graphs = enable ? 1 : 0;
  if (!enable) drop_graphs(b);
  return GWL_OK;
}

int gwl_batcher_eval(gwl_batcher* b, const gwl_batch_item* items, int32_t n, int32_t precision, void* stream) {
  if (!b || (n > 0 && !items) || n < 0) {
    set_error("null argument");
    return GWL_ERR_ARGUMENT;
  }
  if (n == 0) return GWL_OK;
  TraceRange tr("gwl_batcher_eval");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  bool fused = precision == GWL_PRECISION_MIXED;
  for (int q = 0; q < n; ++q) {
    const gwl_batch_item& it = items[q];
    if (!it.analysis || it.B < 0 || (it.B > 0 && (!it.params || !it.out))) {
      set_error("batch item with a null analysis, params or out");
      return GWL_ERR_ARGUMENT;
    }
    const gwl_analysis* a = it.analysis;
    if (a->model != GWL_MODEL_TAYLORF2 || a->time_marg || a->relbin || a->multiband || a->roq ||
        a->n_det > kMultiMaxDet)
      fused = false;
  }
  if (!fused) {
    // other models / precisions / time marginalisation: one launch sequence per item
    for (int q = 0; q < n; ++q) {
      gwl_analysis* a = items[q].analysis;
      std::lock_guard<std::mutex> g(a->mu);
      const int rc = run_eval(a, items[q].params, items[q].B, precision, items[q].out, nullptr, nullptr, s);
      if (rc) return rc;
    }
    return GWL_OK;
  }
  std::lock_guard<std::mutex> g(b->mu);
  // sizes
  int64_t total = 0, n_units = 0;
  size_t part = 0, hist = 0;
  std::vector<LaunchArgs> largs(n);
  std::vector<int64_t> key;
  key.reserve(2 * n + 1);
  key.push_back(n);
  int64_t units_d[kMultiClasses] = {0, 0, 0, 0, 0, 0, 0, 0};  // per kernel class 2 D + cplx
  bool acc_class[kMultiClasses] = {false, false, false, false, false, false, false, false};
  for (int q = 0; q < n; ++q) {
    gwl_analysis* a = items[q].analysis;
    largs[q] = make_args(a, items[q].B, GWL_PRECISION_MIXED);
    ordering_with_marks(largs[q]);
    hist += 2 * (size_t)largs[q].order_keys + 1;
    total += items[q].B;
    part += (size_t)largs[q].n_groups * a->n_det * kPartStride * items[q].B;
    const int64_t tiles = (items[q].B + kPointsPerCta - 1) / kPointsPerCta;
    units_d[2 * a->n_det + largs[q].cplx] += tiles * largs[q].n_groups;
    key.push_back(reinterpret_cast<int64_t>(a));
    key.push_back(items[q].B);
    key.push_back(largs[q].n_groups);  // changes when the analysis is re-tuned
    key.push_back(largs[q].rf_tol > 0);  // the accurate kernel and the histogram layout
    if (largs[q].rf_tol > 0) acc_class[2 * a->n_det + largs[q].cplx] = true;
  }
  for (int c = 0; c < kMultiClasses; ++c) n_units += units_d[c];
  // capacity (growing invalidates captured graphs: their pointers change)
  if (b->staged_pending) {
    GWL_CUDA(cudaEventSynchronize(b->staged));
    b->staged_pending = false;
  }
  const bool need_grow = n > b->cap_items || n_units > b->cap_units || total > b->cap_points || part > b->cap_part ||
                         hist > b->cap_hist;
  if (need_grow) {
    GWL_CUDA(cudaDeviceSynchronize());
    drop_graphs(b);
    int rc;
    if ((rc = grow(&b->d_args, &b->h_args, b->cap_items, (size_t)n))) return rc;
    if ((rc = grow(&b->d_off, &b->h_off, b->cap_items + 1, (size_t)n + 1))) return rc;
    b->cap_items = std::max(b->cap_items, (int)n);
    if ((rc = grow(&b->d_units, &b->h_units, b->cap_units, (size_t)n_units))) return rc;
    b->cap_units = std::max(b->cap_units, n_units);
    if ((rc = grow<PointRec>(&b->d_rec, nullptr, b->cap_points, (size_t)total))) return rc;
    if ((rc = grow<int32_t>(&b->d_order, nullptr, b->cap_points, (size_t)total))) return rc;
    b->cap_points = std::max(b->cap_points, total);
    if ((rc = grow<int32_t>(&b->d_hist, nullptr, b->cap_hist, hist))) return rc;
    b->cap_hist = std::max(b->cap_hist, hist);
    if ((rc = grow<double>(&b->d_part, nullptr, b->cap_part, part))) return rc;
    b->cap_part = std::max(b->cap_part, part);
  }
  // per-item launch arguments, point offsets and work units (grouped by detector count)
  int64_t off = 0;
  size_t poff = 0, hoff = 0;
  int64_t ucur[kMultiClasses + 1];
  int64_t ubeg[kMultiClasses + 1];
  ubeg[0] = 0;
  for (int c = 0; c < kMultiClasses; ++c) ubeg[c + 1] = ubeg[c] + units_d[c];
  for (int c = 0; c <= kMultiClasses; ++c) ucur[c] = ubeg[c];
  for (int q = 0; q < n; ++q) {
    gwl_analysis* a = items[q].analysis;
    LaunchArgs& L = largs[q];
    L.params = items[q].params;
    L.out = items[q].out;
    L.rec = b->d_rec + off;
    L.part = b->d_part + poff;
    L.order = b->d_order + off;
    L.order_hist = b->d_hist + hoff;
    L.rf_count = L.order_hist + 2 * L.order_keys;  // this item's marked points
    hoff += 2 * (size_t)L.order_keys + 1;
    L.status = b->d_status;
    L.rf_total = b->d_counter + 2 * kMultiClasses;
    b->h_args[q] = L;
    b->h_off[q] = off;
    const int64_t tiles = (items[q].B + kPointsPerCta - 1) / kPointsPerCta;
    for (int64_t t = 0; t < tiles; ++t)
      for (int64_t gg = 0; gg < L.n_groups; ++gg)
        b->h_units[ucur[2 * a->n_det + L.cplx]++] = make_int4(q, (int)t, (int)gg, 0);
    off += items[q].B;
    poff += (size_t)L.n_groups * a->n_det * kPartStride * items[q].B;
  }
  b->h_off[n] = off;
  MultiArgs m;
  m.args = b->d_args;
  m.offsets = b->d_off;
  m.n_items = n;
  m.total_points = total;
  m.units = b->d_units;
  for (int c = 0; c <= kMultiClasses; ++c) m.unit_begin[c] = ubeg[c];
  m.counter = b->d_counter;
  m.ordered = 1;
  int ctas[kMultiClasses] = {0, 0, 0, 0, 0, 0, 0, 0};
  int ctas_acc[kMultiClasses] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (int c = 2; c < kMultiClasses; ++c) {
    if (units_d[c] > 0)
      ctas[c] = (int)std::min<int64_t>(units_d[c], (int64_t)sm_count() * multi_tf2_ctas_per_sm(c, false));
    if (units_d[c] > 0 && acc_class[c]) ctas_acc[c] = sm_count() * multi_tf2_ctas_per_sm(c, true);
  }
  auto enqueue = [&]() -> int {
    GWL_CUDA(cudaMemcpyAsync(b->d_args, b->h_args, n * sizeof(LaunchArgs), cudaMemcpyHostToDevice, s));
    GWL_CUDA(cudaMemcpyAsync(b->d_off, b->h_off, (n + 1) * sizeof(int64_t), cudaMemcpyHostToDevice, s));
    GWL_CUDA(cudaMemcpyAsync(b->d_units, b->h_units, n_units * sizeof(int4), cudaMemcpyHostToDevice, s));
    GWL_CUDA(cudaMemsetAsync(b->d_counter, 0, kMultiCounters * sizeof(int), s));
    GWL_CUDA(cudaMemsetAsync(b->d_hist, 0, hoff * sizeof(int32_t), s));
    GWL_CUDA(launch_multi(m, ctas, ctas_acc, s, &b->side));
    return GWL_OK;
  };
  if (b->use_graphs && s != nullptr) {  // the legacy default stream cannot be captured
    auto hit = b->graphs.find(key);
    if (hit == b->graphs.end()) {
      cudaGraph_t graph;
      GWL_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
      const int rc = enqueue();
      cudaError_t ce = cudaStreamEndCapture(s, &graph);
      if (rc) return rc;
      if (ce != cudaSuccess) {
        set_error(std::string("graph capture: ") + cudaGetErrorString(ce));
        return GWL_ERR_CUDA;
      }
      cudaGraphExec_t exec;
      ce = cudaGraphInstantiate(&exec, graph, 0);
      cudaGraphDestroy(graph);
      if (ce != cudaSuccess) {
        set_error(std::string("graph instantiate: ") + cudaGetErrorString(ce));
        return GWL_ERR_CUDA;
      }
      hit = b->graphs.emplace(key, exec).first;
    }
    GWL_CUDA(cudaGraphLaunch(hit->second, s));
  } else {
    const int rc = enqueue();
    if (rc) return rc;
  }
  GWL_CUDA(cudaEventRecord(b->staged, s));
  b->staged_pending = true;
  return GWL_OK;
}

int gwl_batcher_last_refined(gwl_batcher* b, void* stream, int64_t* count) {
  if (!b || !count) {
    set_error("null argument");
    return GWL_ERR_ARGUMENT;
  }
  *count = 0;
  std::lock_guard<std::mutex> g(b->mu);
  if (!b->d_counter) return GWL_OK;
  int n = 0;
  GWL_CUDA(cudaStreamSynchronize(static_cast<cudaStream_t>(stream)));
  GWL_CUDA(cudaMemcpy(&n, b->d_counter + 2 * kMultiClasses, sizeof(int), cudaMemcpyDeviceToHost));
  *count = n;
  return GWL_OK;
}

int gwl_selftest_bounded_wait(uint32_t poll_limit, void* stream, int* device_status, int* arrived) {
  if (!device_status || !arrived || poll_limit == 0) {
    set_error("null argument or zero poll limit");
    return GWL_ERR_ARGUMENT;
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int* d = nullptr;
  GWL_CUDA(cudaMalloc(&d, 2 * sizeof(int)));
  cudaError_t e = cudaMemsetAsync(d, 0, 2 * sizeof(int), s);
  if (e == cudaSuccess) e = launch_wait_selftest(poll_limit, d, d + 1, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(device_status, d, sizeof(int), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(arrived, d + 1, sizeof(int), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  cudaFree(d);
  if (e != cudaSuccess) {
    set_error(std::string("gwl_selftest_bounded_wait: ") + cudaGetErrorString(e));
    return GWL_ERR_CUDA;
  }
  if (*device_status == kDevStatusTimeout) {
    set_error("a bounded device wait gave up (bulk copy did not complete)");
    return GWL_ERR_TIMEOUT;
  }
  return GWL_OK;
}

int gwl_inject_device_status(gwl_analysis* a, int value) {
  if (!a) {
    set_error("null argument");
    return GWL_ERR_ARGUMENT;
  }
  std::lock_guard<std::mutex> g(a->mu);
  GWL_CUDA(cudaMemcpyAsync(a->d_status, &value, sizeof(int), cudaMemcpyHostToDevice, a->stream));
  GWL_CUDA(cudaStreamSynchronize(a->stream));
  return GWL_OK;
}

int gwl_batcher_status(gwl_batcher* b, int* device_status) {
  if (!b || !device_status) {
    set_error("null argument");
    return GWL_ERR_ARGUMENT;
  }
  GWL_CUDA(cudaMemcpy(device_status, b->d_status, sizeof(int), cudaMemcpyDeviceToHost));
  if (*device_status) cudaMemset(b->d_status, 0, sizeof(int));
  return GWL_OK;
}

int gwl_distance_lookup_table(const double* distance, const double* prior, int32_t n, double ref_dist,
                              const double* dh_axis, int32_t n_dh, const double* hh_axis, int32_t n_hh,
                              int phase_marginalization, double* table) {
  if (!distance || !prior || !dh_axis || !hh_axis || !table || n < 2 || n_dh < 1 || n_hh < 1 || !(ref_dist > 0)) {
    set_error("invalid lookup-table arguments");
    return GWL_ERR_ARGUMENT;
  }
  const double dd = distance[1] - distance[0];
  std::vector<double> sc(n), sc2(n), wt(n);
  KahanSum norm;
  for (int k = 0; k < n; ++k) {
    sc[k] = ref_dist / distance[k];
    sc2[k] = sc[k] * sc[k];
    wt[k] = prior[k] * dd;
    norm.add(wt[k]);
  }
  // logsumexp(0 / d, b = prior * dd) = log(sum b)
  const double log_norm = std::log(norm.value());
  double *d_dh = nullptr, *d_hh = nullptr, *d_sc = nullptr, *d_sc2 = nullptr, *d_wt = nullptr, *d_li = nullptr,
         *d_tab = nullptr;
  int rc = GWL_OK;
  cudaError_t e;
  const size_t tab = (size_t)n_dh * n_hh;
  if ((e = cudaMalloc(&d_dh, n_dh * sizeof(double))) != cudaSuccess) goto cuda_fail;
  if ((e = cudaMalloc(&d_hh, n_hh * sizeof(double))) != cudaSuccess) goto cuda_fail;
  if ((e = cudaMalloc(&d_sc, n * sizeof(double))) != cudaSuccess) goto cuda_fail;
  if ((e = cudaMalloc(&d_sc2, n * sizeof(double))) != cudaSuccess) goto cuda_fail;
  if ((e = cudaMalloc(&d_wt, n * sizeof(double))) != cudaSuccess) goto cuda_fail;
  if ((e = cudaMalloc(&d_tab, tab * sizeof(double))) != cudaSuccess) goto cuda_fail;
  if (phase_marginalization && (e = cudaMalloc(&d_li, (size_t)n_dh * n * sizeof(double))) != cudaSuccess)
    goto cuda_fail;
  if ((e = cudaMemcpy(d_dh, dh_axis, n_dh * sizeof(double), cudaMemcpyHostToDevice)) != cudaSuccess) goto cuda_fail;
  if ((e = cudaMemcpy(d_hh, hh_axis, n_hh * sizeof(double), cudaMemcpyHostToDevice)) != cudaSuccess) goto cuda_fail;
  if ((e = cudaMemcpy(d_sc, sc.data(), n * sizeof(double), cudaMemcpyHostToDevice)) != cudaSuccess) goto cuda_fail;
  if ((e = cudaMemcpy(d_sc2, sc2.data(), n * sizeof(double), cudaMemcpyHostToDevice)) != cudaSuccess) goto cuda_fail;
  if ((e = cudaMemcpy(d_wt, wt.data(), n * sizeof(double), cudaMemcpyHostToDevice)) != cudaSuccess) goto cuda_fail;
  if ((e = launch_distance_table(d_dh, n_dh, d_hh, n_hh, d_sc, d_sc2, d_wt, n, d_li, phase_marginalization, log_norm,
                                 d_tab)) != cudaSuccess)
    goto cuda_fail;
  if ((e = cudaMemcpy(table, d_tab, tab * sizeof(double), cudaMemcpyDeviceToHost)) != cudaSuccess) goto cuda_fail;
  goto done;
cuda_fail:
  set_error(std::string("distance lookup table: ") + cudaGetErrorString(e));
  rc = GWL_ERR_CUDA;
done:
  cudaFree(d_dh);
  cudaFree(d_hh);
  cudaFree(d_sc);
  cudaFree(d_sc2);
  cudaFree(d_wt);
  cudaFree(d_li);
  cudaFree(d_tab);
  return rc;
}

int gwl_host_math(int what, const double* x, const double* y, int64_t n, const double* tx, int32_t nx,
                  const double* ty, int32_t ny, const double* c, const double bbox[4], double* out) {
  if (!x || !out || n < 0) {
    set_error("null argument");
    return GWL_ERR_ARGUMENT;
  }
  if (what == 0) {
    for (int64_t i = 0; i < n; ++i) out[i] = gwl::ln_i0(x[i]);
    return GWL_OK;
  }
  if (what == 1) {
    if (!y || !tx || !ty || !c || !bbox || nx < 8 || ny < 8) {
      set_error("spline evaluation needs knots, coefficients and a box");
      return GWL_ERR_ARGUMENT;
    }
    for (int64_t i = 0; i < n; ++i) out[i] = gwl::bicubic_eval(tx, nx, ty, ny, c, bbox, x[i], y[i]);
    return GWL_OK;
  }
  set_error("unknown host_math selector");
  return GWL_ERR_ARGUMENT;
}

}  // extern "C"
