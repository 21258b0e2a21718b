// Internal declarations shared by the host runtime (gwl_capi.cu) and the
// kernel translation units.  Not part of the public ABI (include/gwlnl.h).
#pragma once

#include <cstddef>
#include <cstdint>
#include <string>

#include <cuda_runtime.h>

#include "../../include/gwlnl.h"

namespace gwl {

constexpr int kMaxDet = GWL_MAX_DETECTORS;
constexpr int kPointsPerCta = 128;     // one thread per parameter point
constexpr int kChunkPlain = 256;       // bins per CTA, float64 kernels
constexpr int kChunkMixed = 512;       // bins per CTA, mixed-precision kernels
constexpr int kBinAlign = 16;          // chunk starts are multiples of this many bins
constexpr int kNumBasis = 8;           // TaylorF2 phase basis functions of f
constexpr int kPartStride = 6;         // partial-sum components per (group, detector, point)
constexpr int kAnchorStep = 8;         // bins between TaylorF2 phase anchors in the table
constexpr int kAnchorOrders = 7;       // Taylor orders 0..6 of the phase about an anchor
constexpr int kAnchorFF = 4;           // orders 0..3 kept in float-float
constexpr int kAnchorFloats = 96;      // per anchor: hi[7][8], lo[4][8], padding
constexpr int kChunksPerGroup = 4;     // chunks walked by one split-K CTA of the TaylorF2 mixed kernel
constexpr int kOrderMaxKeys = 4096;    // buckets of the point ordering by band end
constexpr int kDevStatusOk = 0;
constexpr int kDevStatusTimeout = 1;
constexpr int kDevStatusBadInput = 2;
constexpr int kDevStatusIndex = 3;  // checked builds (-DGWL_CHECK): an index check failed, the access was skipped
constexpr uint32_t kWaitLimit = 1u << 22;  // polls of a bulk-copy barrier before giving up
// Refinement of the TaylorF2 mixed-precision result (see LaunchArgs::rf_tol):
// the error bound of a point is kRefineL2 * L2 + kRefineL1 * L1, with L2 the
// Euclidean norm of its per-bin terms |<d|h>_k| and L1 their sum over the
// bins where the data are signal-dominated (whitened power 4 |d|^2 / (T S)
// above kRefineLoudPower).  The coefficients hold with a margin of 2.5 to 4
// over the measured error of the fast kernel on short, loud analyses.
constexpr double kRefineL2 = 1e-6;
constexpr double kRefineL1 = 1e-7;
constexpr double kRefineLoudPower = 10.0;
constexpr double kRefineDefaultTol = 5e-4;
constexpr int kCosTable = 1024;        // angles of the float-float cos / sin table of the accurate kernel
constexpr int kRoqSplits = 8;          // node groups of the mixed ROQ time-marginalised matrix products

// Per-point quantities computed once per evaluation by the float64 prologue.
struct PointRec {
  double fp[kMaxDet], fx[kMaxDet], dt[kMaxDet];  // antenna patterns; (t_geo - t_start) + delay
  uint32_t xfix[kMaxDet][2];                     // frac(dt * df) as 0.64 fixed point {lo, hi}
  uint32_t qfix[kMaxDet][2];                     // TaylorF2 real-part kernel: arg(conj(Q_d)) / 2 pi, 0.64 fixed
  double qabs[kMaxDet];                          // |Q_d|, Q_d = Fp (1 + cos^2 i) / 2 - i Fx cos i
  double amp;          // TaylorF2 amplitude prefactor A0 | sine-Gaussian plus factor
  double amp2;         // sine-Gaussian cross factor
  double sg_f0, sg_a;  // sine-Gaussian centre frequency, pi^2 tau^2
  double m_sec, eta, f_isco, cos_i, phase, dist, jitter;
  double a[8], l[8];                 // TaylorF2 phase coefficients
  float c_hi[kNumBasis + 1];         // TaylorF2 phase basis coefficients in cycles (float-float)
  float c_lo[kNumBasis + 1];         // index kNumBasis: frac of the constant term
  int64_t k_start, k_end;            // TaylorF2 band [k_start, k_end) on the analysis grid
  int32_t valid;                     // 0: waveform undefined (lnL = nan_to_num(-inf))
  int32_t refine;                    // TaylorF2 mixed: error bound above the tolerance (LaunchArgs::rf_tol)
  // mixed time-marginalised kernel over the full grid (k_time_marg): per-point
  // scalars from the float64 prologue, so that the kernel runs no float64 per
  // point before its transform nor per time sample
  float tm_coef[2 * kMaxDet];        // detector response coefficients of the integrand
  double tm_hh;                      // TaylorF2 <h|h>
  int64_t tm_j0, tm_j1;              // FFT indices of the first and last time sample inside the prior
  int32_t tm_row_ly, tm_row_in;      // TaylorF2 with the distance table: the spline's row at this <h|h>
  float tm_row_hy[4];                // (SplineRowF: interval, inside the table, basis values)
  float tm_xp, tm_zs;                // the kernel's largest |X| over the window and ||z||_2, for the error bound
};

// Relative binning, per grid index: its bin and the offset of its frequency
// from the bin's centre.
struct RbBinF {
  int32_t bin;
  float x;
};

struct DetGeom {
  double vertex[3];
  double tensor[9];
  double start_time;
};

// Everything a kernel needs, passed by value.
struct LaunchArgs {
  int model, n_det, precision;
  int cplx;                             // TaylorF2 mixed: 1 = complex <d|h> partials, 0 = real part only
  int64_t B;
  int64_t n_bins, k_lo, k_hi, k_base;   // in-band hull [k_lo, k_hi); chunk origin k_base
  int64_t n_chunks;                     // chunks over [k_base, k_hi)
  int64_t n_groups;                     // CTAs along the bin axis; CTA g walks chunks g, g + G, ...
  int chunk;                            // bins per chunk
  double duration, step, fmin;
  int64_t k_fmin;                       // first bin with f >= minimum_frequency
  DetGeom det[kMaxDet];
  const double* freq;                   // [n_pad] float64 frequency array
  const float* freq_f;                  // [n_pad] float32 copy (sine-Gaussian mixed)
  const double* strain[kMaxDet];        // [2*n_pad] masked strain
  const double* inv_psd[kMaxDet];       // [n_pad] mask / S
  const float2* w[kMaxDet];             // [n_pad] mixed data weights (scaled)
  const uint2* wp[kMaxDet];             // [n_pad] TaylorF2: polar weights {float |w| bits, arg(w) 0.32 cycles}
  const uint4* wq[kMaxDet];             // [n_pad / 2] TaylorF2 fast kernel: per bin pair {|w| even, |w| odd,
                                        // tau even, tau odd}, tau = arg(w) at bins k % 8 == 0, else
                                        // arg(w_k) - arg(w_{k-1}) (0.32 cycles, wrapping)
  const float* v[kMaxDet];              // [n_pad] mixed inverse PSD (scaled)
  const float* v_lo[kMaxDet];           // [n_pad] sine-Gaussian: low words of the scaled inverse PSD (v + v_lo)
  const double* hh_prefix[kMaxDet];     // [n_bins + 1] TaylorF2 <h|h> prefix sums
  double w_scale[kMaxDet], v_scale[kMaxDet];
  const float2* basis;                  // [n_pad][kNumBasis] float-float phase basis
  const double4* ftab;                  // [n_pad] {f^(1/3), ln(f) / 3, f^(-5/3), f^(-7/6)} (float64 TaylorF2)
  const float* anchors;                 // [n_anchors][kAnchorFloats] Taylor tables of the basis
  int64_t n_anchors;
  const double* params;                 // [GWL_NPARAM][B]
  PointRec* rec;                        // [B]
  double* part;                         // [n_groups][n_det][kPartStride][B] (point fastest)
  double* out;                          // [B]
  double* dh_out;                       // optional [2B] complex <d|h> totals
  double* hh_out;                       // optional [B] <h|h> totals
  int* status;                          // device status word
  // error control of the TaylorF2 mixed-precision sums: the prologue bounds
  // each point's error from the prefix sums rf_p2 (|w|^2) and rf_p1 (|w| over
  // signal-dominated bins); a point whose bound exceeds rf_tol is marked
  // (PointRec::refine), counted in rf_count and ordered into the first slots,
  // which the accurate variant of the bin-walking kernel evaluates (float-float
  // cosine from cos_tab, TwoSum accumulation per bin).  rf_tol <= 0: off.
  const double* rf_p2[kMaxDet];         // [n_bins + 1]
  const double* rf_p1[kMaxDet];         // [n_bins + 1]
  double rf_tol;
  int* rf_count;                        // marked points of this analysis (zeroed with the ordering histogram)
  int* rf_total;                        // optional: marked points of the whole launch
  const float4* cos_tab;                // [kCosTable] {cos hi, cos lo, sin hi, sin lo} of 2 pi q / kCosTable
  // optional point ordering (TaylorF2 mixed): thread slot s of the bin-walking
  // kernel evaluates point order[s]; points are grouped by the chunk that
  // holds their band end, longest first, so that the 128 points of a CTA stop
  // at nearly the same bin.  nullptr: slot s evaluates point s.
  int32_t* order;                       // [B]
  int32_t* order_hist;                  // [2 * order_keys]: counts (then bases), cursors; zeroed before use
  int order_keys, order_shift;
  int order_half;                       // keys of marked points (PointRec::refine) are offset by this
  // marginalisation
  int time_marg, phase_marg, dist_marg, jitter;
  double t_min, t_max, delta_tc, start_time0;
  double tm_step, tm_inv_step, tm_prob, inv_ref_dist;  // T / L, L / T, 1 / (t_max - t_min), 1 / ref_dist
  int64_t n_fft;                        // time-marginalisation FFT length (n_bins - 1)
  const double* tx; const double* ty; const double* tc;  // distance spline
  const float* tx_f; const float* ty_f; const float* tc_f; // float32 copy (mixed precision)
  float bbox_x_f[2];                    // bbox[0] rounded up and bbox[1] rounded down to float32: the same
                                        // test of a float32 x as against the float64 bounds
  int nx, ny;
  double bbox[4];
  double ref_dist;
  double* tm_work;                      // time-marginalisation work space
  double* tm_series;                    // optional [B][2 n_fft] FFT of the integrand (float64 kernel)
  int tm_first;                         // time of FFT index j: start + (j + tm_first) * duration / n_fft
  int antenna_fixed;                    // antenna patterns at antenna_time instead of geocent_time
  double antenna_time;
  // relative binning: the model at the bin edges, its ratio to the fiducial
  // response, and the per-bin summary data of each detector
  int relbin;
  int rb_edges;
  const int64_t* rb_index;              // [rb_edges] grid index of each edge
  const double* rb_freq;                // [rb_edges] edge frequencies
  const double2* rb_h0inv[kMaxDet];     // [rb_edges] 1 / h0_d(f_e)
  const double* rb_sum[kMaxDet];        // [rb_edges - 1][6]: a0 re, a0 im, a1 re, a1 im, b0, b1
  // relative binning with time marginalisation: the full-grid weights
  // 4/T h0_d(f) conj(d(f)) / S(f) and the bin of each grid index in
  // [rb_index[0], rb_index[rb_edges - 1]]
  const double2* rb_g[kMaxDet];         // [n_bins]
  const int32_t* rb_bin;                // [rb_index[last] - rb_index[0] + 1]
  // ... and for the mixed-precision kernel over the same span: the weights in
  // float32 and, per grid index, its bin with f - (f_b + f_b+1) / 2
  const float2* rb_gf[kMaxDet];         // [rb_index[last] - rb_index[0] + 1]
  const RbBinF* rb_bx;                  // [rb_index[last] - rb_index[0] + 1]
  int tw_refine_only;                   // float64 windowed time marginalisation: only the marked points
  float2* tw_scratch;                   // mixed windowed multi-banding: [tw_scratch_slots][mb_points] banded values
  int64_t tw_scratch_slots;
  int32_t* rf_list;                     // windowed mixed kernel: the marked points, [*rf_count]
  double* tw_part;                      // float64 recomputation: [tw_part_units][n_win_max + 1] complex shares
  int* tw_done;                         // ... finished units per marked point, [tw_part_units], zeroed before
  int64_t tw_part_units;
  // multi-banding: the model at the banded frequencies, weighted by the
  // per-detector linear (complex) and quadratic (real) coefficients
  int multiband;
  int64_t mb_points;
  const double* mb_freq;                // [mb_points] banded frequencies
  const double4* mb_pow;                // [mb_points] {f^(1/3), ln(f) / 3, f^(-5/3), f^(-7/6)}
  const double2* mb_lin[kMaxDet];       // [mb_points]
  const double* mb_quad[kMaxDet];       // [mb_points]
  int mb_bands;
  const int64_t* mb_band_start;         // [mb_bands + 1] first banded index of each band (and the end)
  const double* mb_band_df;             // [mb_bands] frequency spacing of each band
  // mixed precision: the float-float phase basis at the banded frequencies, the
  // linear coefficients times f^(-7/6) in float32 (scaled by mb_lw_scale), and
  // prefix sums of f^(-7/3) times the quadratic coefficients
  const float2* mb_basis;               // [mb_points][kNumBasis]
  const float2* mb_lw[kMaxDet];         // [mb_points]
  double mb_lw_scale[kMaxDet];
  // time marginalisation with a prior other than Uniform: its density on the
  // nodes t0 + g h (g < tm_prior_n, h a power of two), read by 4-node Lagrange
  // interpolation; tm_prior == nullptr means the Uniform density tm_prob
  const double* tm_prior;
  const float* tm_prior_f;
  int64_t tm_prior_n;
  double tm_prior_t0, tm_prior_inv_h;
  const double* mb_qprefix[kMaxDet];    // [mb_points + 1]
  const double* mb_l2prefix[kMaxDet];   // [mb_points + 1] prefix sums of |mb_lw|^2 (error bound of the mixed kernel)
  int mb_refine_only;                   // float64 multi-banding kernel: only the points marked by the mixed one
  // multi-banding with time marginalisation: for each full-resolution index
  // k < n_fft the banded points scattered there, mb_tm_src[mb_tm_ptr[k] ..
  // mb_tm_ptr[k + 1]); a code c >= 0 is banded point c, c < 0 is banded point
  // -c - 1 counted in <h|h> only (replaced at its index within its band)
  int mb_tm;
  const int32_t* mb_tm_ptr;             // [n_fft + 1]
  const int32_t* mb_tm_src;             // [mb_points]
  // multi-banding with the IFFT-FFT <h|h> (multiband.py:613-650, 760-779):
  // the odd-bin part of band b >= 1 of detector d at point i,
  // mb_fft_hh[(b * n_det + d) * B + i], written by k_mb_hh_fft before the
  // kernels that add it to <h|h> (band 0 is wholly in mb_quad); null without it
  const double* mb_fft_hh;
  // distance marginalisation without time marginalisation: a bound r_max =
  // d_ref / d_min on the lnL's slope E[d_ref / d] in <d|h> (and r_max^2 / 2 in
  // <h|h>), by which the mixed kernels scale their error bounds; values <= 1
  // (no distance table, or time marginalisation with its own sensitivities)
  // leave them as they are
  double dist_slope;
  // reduced-order quadrature: the model at the linear and quadratic nodes,
  // time-dependent linear weights on the grid (t_start + k) dt, k < n_time
  int roq;
  int roq_nl, roq_nq;
  int64_t roq_time_start, roq_n_time;
  double roq_dt;
  const double* roq_fl;                 // [roq_nl] linear nodes
  const double* roq_fq;                 // [roq_nq] quadratic nodes
  const double4* roq_pl;                // [roq_nl] TaylorF2 powers of the linear nodes
  const double4* roq_pq;                // [roq_nq] and of the quadratic nodes
  const double2* roq_wl[kMaxDet];       // [roq_n_time][roq_nl]
  const double* roq_wq[kMaxDet];        // [roq_nq]
  // ROQ with time marginalisation (roq.py:320-331, 535-541, 604-651): the
  // regular time grid of the marginalisation and the most weight rows one
  // point reads per detector; the prologue then stores in dt[d] the detector's
  // delay at antenna_time alone
  int roq_tm;
  int64_t roq_tm_n, roq_tm_chunk, roq_tm_rows;  // samples, samples per chunk, rows per chunk (at most)
  const double* roq_tm_times;           // [roq_tm_n]
  // ... in mixed precision, over one chunk of points [roq_c0, roq_c0 + roq_cn):
  // conj(h_d) at the linear nodes in float32, complex float32 matrix
  // products per detector over every weight row, the nodes split into
  // kRoqSplits groups of roq_ks (roq_d32[d][s] = roq_wl32 h over group s),
  // then per point the groups' sums in float-float and the per-sample
  // interpolation and marginalisation in float32
  const float2* roq_wl32[kMaxDet];      // [roq_n_time][roq_nl_pad] float32 copy of roq_wl, zero-padded
  float roq_wnorm[kMaxDet][kRoqSplits]; // per node group: largest Euclidean norm of a row of roq_wl
  int roq_nl_pad, roq_ks;               // kRoqSplits * roq_ks nodes (padded), roq_ks per group
  const int2* roq_tm_g;                 // [roq_tm_n] (t_j - start_0 - t_grid0) / dt: {floor, float fraction bits}
  float2* roq_h32;                      // [n_det][roq_cn][roq_nl_pad]
  float2* roq_d32;                      // [n_det][kRoqSplits][roq_cn][roq_n_time]
  double* roq_hh;                       // [roq_cn] <h|h>
  int64_t roq_c0, roq_cn;
  int rf_list_only;                     // float64 ROQ time marginalisation of the listed points alone
};

// A batch over several analyses evaluated by one persistent launch: per item
// (one analysis and its points) a LaunchArgs; work units (item, point tile,
// chunk group) are pulled by the persistent CTAs from an atomic counter.
struct MultiArgs {
  const LaunchArgs* args;   // [n_items]
  const int64_t* offsets;   // [n_items + 1] first global point of each item
  int n_items;
  int64_t total_points;
  const int4* units;        // [n_units] {item, tile, group, 0}, grouped by kernel class
  int64_t unit_begin[9];    // units of class q = 2 D + cplx: [unit_begin[q], unit_begin[q + 1])
  int* counter;             // [kMultiCounters], zeroed before the launch: units taken per class by the
                            // fast kernels, then by the accurate kernels, then the marked points
  int ordered;              // items carry a point ordering (LaunchArgs::order)
};

// One compiled prior (gwl_priors_create): device copy of a gwl_prior with
// device table pointers.
struct PriorEntry {
  int kind, target, column, table_n;
  double p[4];
  const double* x;
  const double* y;
};

// A second, high-priority stream on which the accurate kernel runs beside the
// fast one: forked from the launching stream after the ordering and joined
// before the reduction (both capturable in a CUDA graph).
struct SideStream {
  cudaStream_t stream = nullptr;
  cudaEvent_t fork = nullptr, join = nullptr;
};
cudaError_t side_stream_create(SideStream* s);
void side_stream_destroy(SideStream* s);
cudaError_t side_fork(SideStream& side, cudaStream_t s);   // side waits for the work enqueued so far on s
cudaError_t side_join(SideStream& side, cudaStream_t s);   // s waits for the work enqueued so far on side

// Kernel launchers (defined in gwl_kernels.cu / gwl_marg.cu).
constexpr int kMultiMaxDet = 3;
constexpr int kMultiClasses = 2 * (kMultiMaxDet + 1);  // kernel class q = 2 * detectors + cplx
constexpr int kMultiCounters = 2 * kMultiClasses + 1;  // unit counters (fast, accurate), then the marked points
cudaError_t launch_multi(const MultiArgs& m, const int* ctas, const int* ctas_acc, cudaStream_t s, SideStream* side);
int multi_tf2_ctas_per_sm(int q, bool acc);
cudaError_t launch_prologue(const LaunchArgs& a, cudaStream_t s);
cudaError_t launch_plain(const LaunchArgs& a, cudaStream_t s);
cudaError_t launch_mixed(const LaunchArgs& a, cudaStream_t s);
// The accurate kernel for the marked points (nothing when rf_tol <= 0).
cudaError_t launch_mixed_acc(const LaunchArgs& a, cudaStream_t s);

cudaError_t launch_finalize(const LaunchArgs& a, cudaStream_t s);
cudaError_t launch_sg_refine(const LaunchArgs& a, cudaStream_t s);
cudaError_t launch_order(const LaunchArgs& a, cudaStream_t s);
cudaError_t launch_relbin(const LaunchArgs& a, cudaStream_t s);
cudaError_t launch_multiband(const LaunchArgs& a, cudaStream_t s);
cudaError_t launch_multiband_mixed(const LaunchArgs& a, cudaStream_t s);
cudaError_t launch_roq(const LaunchArgs& a, cudaStream_t s);
cudaError_t launch_roq_time_marginalized(const LaunchArgs& a, cudaStream_t s);
// Mixed ROQ time marginalisation of one chunk: the node values before the
// matrix products, the interpolation and marginalisation after them.
constexpr int64_t kRoqMixedChunk = 1024;  // points per chunk
// whether the mixed kernel's shared memory (rows of every detector, spline knots) fits
bool roq_tm_mixed_fits(const LaunchArgs& a);
cudaError_t launch_roq_nodes32(const LaunchArgs& a, cudaStream_t s);
cudaError_t launch_roq_tm_mixed(const LaunchArgs& a, cudaStream_t s);
void order_layout(int64_t n_chunks, int* keys, int* shift);
// Ordering of a mixed TaylorF2 launch: the band-end keys, doubled when points
// can be marked for the accurate kernel (rf_tol > 0; their keys take the upper
// half); the marked count follows the 2 * order_keys histogram words (zeroed
// with them: 2 * order_keys + 1 words in all).  order_hist, if set, must hold them.
void ordering_with_marks(LaunchArgs& L);
void ordering_by_peak(LaunchArgs& L);
cudaError_t launch_time_marginalized(const LaunchArgs& a, cudaStream_t s);
// The mixed full-grid time-marginalised kernel's error bounds, from what it
// stored in the point records: marks the points over the tolerance.
cudaError_t launch_time_marg_marks(const LaunchArgs& a, cudaStream_t s);
// Relative binning / multi-banding with time marginalisation by the windowed
// four-step transform (gwl_marg_window.cu): whether this launch's shared
// memory fits, and the launch (mixed precision: relative binning only).
bool time_marg_window_fits(const LaunchArgs& a);
bool time_marg_window_mixed_ready(const LaunchArgs& a);  // the mixed kernel's tables and work space are there
bool time_marg_window_refine_fits(const LaunchArgs& a);  // the float64 recomputation of marked points fits
int64_t time_marg_window_slots();                        // work-space slots of the mixed multi-banding kernel
// bytes per unit of the float64 recomputation's shares (0: the window does not fit)
size_t time_marg_window_share_bytes(const LaunchArgs& a);
cudaError_t launch_time_marg_window(const LaunchArgs& a, cudaStream_t s);
// FFT lengths the time-marginalised kernels take: L = m 2^p with m odd,
// m <= kTmMaxOddFactor and p >= 4 (m and p returned)
constexpr int kTmMaxOddFactor = 127;
bool fft_length_supported(int64_t L, int* m_odd, int* log2N);
size_t time_marg_work_bytes(const LaunchArgs& a);
// Multi-banding with the IFFT-FFT <h|h> (gwl_mb_fft.cu): one band's odd-bin
// transform.  Transforms of at most 2^kMbFftSmemLog2 samples run in shared
// memory, longer ones in a global slot of 2^log2m double2 per CTA.
constexpr int kMbFftSmemLog2 = 13;
struct MbFftBand {
  int band;                      // b >= 1
  int ks;                        // K_s: grid index of the band's first banded point
  int log2m;                     // M = Mbs[b] = 2^log2m samples
  int log2m_max;                 // twiddle table length 2^log2m_max >= M
  int in_smem;                   // 1: the transform in shared memory
  double scale;                  // 4 / That_b
  const double* odd[kMaxDet];    // [M / 2] Re I_(2j+1) of each detector
  const double* sqrtw;           // [mb_points] square roots of the band windows
  const double2* tw;             // [2^(log2m_max + 1)] exp(-i pi k / 2^log2m_max)
  double* out;                   // the mb_fft_hh slab
  // float64 kernel: only the listed points (list_count of them), or all
  const int32_t* list;
  const int32_t* list_count;
  // float32 kernel (TaylorF2, mixed precision): the twiddles in float32, the
  // banded amplitude table sqrt(w_k) f_k^(-7/6) / aw_scale, and the error slab
  // (same layout as out)
  const float2* tw32;
  const float* aw;
  double aw_scale;
  const float2* odd32[kMaxDet];  // [M / 2] float-float Re I_(2j+1) / odd32_scale
  double odd32_scale;            // the band's largest |Re I_(2j+1)|
  double* err;
};
size_t mb_hh_fft_smem(int log2m);  // dynamic shared memory of a float64 transform in shared memory, 0 if it does not fit
bool mb_hh_fft32_in_smem(int log2m);
// one band's transforms: float64 (mixed = false; all points or the listed
// ones) or float32 with the error bound (mixed = true); scratch holds
// scratch_slots slots of 2^log2m complex values of that precision
cudaError_t launch_mb_hh_fft(const LaunchArgs& a, const MbFftBand& band, void* scratch, int64_t scratch_slots,
                             bool mixed, cudaStream_t s);
// the points whose float32 error, summed over bands and detectors, exceeds tol
cudaError_t launch_mb_fft_marks(const LaunchArgs& a, const double* err, double tol, int32_t* list, int32_t* count,
                                cudaStream_t s);
cudaError_t launch_source_polarizations(int model, const double* freq, int64_t n, const double* params,
                                        double fmin, double* plus, double* cross, cudaStream_t s);
cudaError_t launch_detector_response(const DetGeom& g, const double* freq, int64_t n, const double* plus,
                                     const double* cross, const double* params, double* resp, cudaStream_t s);

cudaError_t launch_distance_table(const double* dh_axis, int n_dh, const double* hh_axis, int n_hh,
                                  const double* scaling, const double* scaling2, const double* weight, int n,
                                  double* lni0_work, int phase, double log_norm, double* table);
cudaError_t launch_wait_selftest(uint32_t limit, int* status, int* arrived, cudaStream_t s);

void set_error(const std::string& msg);
int noalloc_launch_args(gwl_analysis* a, int64_t B, LaunchArgs* L, size_t* rec_bytes, size_t* part_bytes);

}  // namespace gwl
