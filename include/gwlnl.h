/*
 * gwlnl.h -- C ABI of the GB300 gravitational-wave transient likelihood.
 *
 * One analysis handle holds, resident in device memory, everything that
 * bilby's GravitationalWaveTransient reads from its Interferometer objects
 * (masked strain, PSD, frequency mask, detector geometry) plus the tables the
 * kernels derive from them.  A batch call evaluates log_likelihood_ratio for
 * B parameter points in one fused launch sequence; the strain h(f) is never
 * written to device memory.
 *
 * The entry points replace, for the sine-Gaussian and TaylorF2 source models
 * and identity calibration, the reference call chain
 *
 *   GravitationalWaveTransient.__init__          bilby/gw/likelihood/base.py:150-229
 *   GravitationalWaveTransient.noise_log_likelihood  base.py:402-417
 *   GravitationalWaveTransient.log_likelihood_ratio  base.py:419-477
 *     -> WaveformGenerator.frequency_domain_strain   bilby/gw/waveform_generator.py:113-209
 *     -> Interferometer.get_detector_response        bilby/gw/detector/interferometer.py:303-368
 *     -> noise_weighted_inner_product                bilby/gw/utils.py:118-138
 *     -> time / phase / distance marginalisation     base.py:775-820
 *
 * Conventions: every function returns a gwl_status (0 = success); no C++
 * exception crosses the ABI; gwl_last_error() returns a description of the
 * last failure on the calling thread.  Arrays are plain pointers with
 * explicit sizes; complex arrays are interleaved (re, im) float64.
 * One handle is used by one host thread at a time.
 */
#ifndef GWLNL_H
#define GWLNL_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  GWL_OK = 0,
  GWL_ERR_ARGUMENT = 1,      /* invalid argument (maps to ValueError) */
  GWL_ERR_CUDA = 2,          /* a CUDA runtime call failed */
  GWL_ERR_MEMORY = 3,        /* device allocation failed or HBM budget exceeded */
  GWL_ERR_UNSUPPORTED = 4,   /* model / option not implemented (NotImplementedError) */
  GWL_ERR_TIMEOUT = 5,       /* a bounded device wait gave up */
  GWL_ERR_STATE = 6,         /* handle not configured for the request */
  GWL_ERR_CHECK = 7          /* checked builds (-DGWL_CHECK): a device index check failed */
} gwl_status;

typedef enum {
  GWL_MODEL_SINEGAUSSIAN = 1, /* bilby/gw/source.py:1153-1209 */
  GWL_MODEL_TAYLORF2 = 2      /* 3.5PN aligned-spin TaylorF2 (published PN phase) */
} gwl_model;

typedef enum {
  GWL_PRECISION_FP64 = 0,  /* plain fused float64 kernels: the drop-in */
  GWL_PRECISION_MIXED = 1  /* float-float phase + fixed-point time shift, float32 products */
} gwl_precision;

/* Parameter slots of the [GWL_NPARAM][B] float64 parameter block. */
typedef enum {
  GWL_P_RA = 0,
  GWL_P_DEC,
  GWL_P_PSI,
  GWL_P_GEOCENT_TIME,
  GWL_P_TIME_JITTER,
  GWL_P_HRSS,
  GWL_P_Q,
  GWL_P_FREQUENCY,
  GWL_P_MASS_1,
  GWL_P_MASS_2,
  GWL_P_CHI_1,
  GWL_P_CHI_2,
  GWL_P_LUMINOSITY_DISTANCE,
  GWL_P_THETA_JN,
  GWL_P_PHASE,
  GWL_NPARAM
} gwl_param;

#define GWL_MAX_DETECTORS 4

/* One Interferometer, as the likelihood reads it
 * (interferometer.py:551-564, strain_data.py:143-233, detector/geometry.py:201-270). */
typedef struct {
  char name[8];
  double vertex[3];        /* geometry.vertex, metres, geocentric */
  double tensor[9];        /* geometry.detector_tensor, row major */
  double start_time;       /* strain_data.start_time (GPS s) */
  const double *strain;    /* [2*n_bins] masked frequency_domain_strain, host */
  const double *psd;       /* [n_bins] power_spectral_density_array, host (+inf allowed) */
  const uint8_t *mask;     /* [n_bins] frequency_mask, host */
} gwl_detector;

typedef struct {
  int32_t model;               /* gwl_model */
  int32_t n_detectors;         /* 1..GWL_MAX_DETECTORS */
  int64_t n_bins;              /* len(frequency_array) */
  double duration;             /* waveform_generator.duration */
  double sampling_frequency;   /* waveform_generator.sampling_frequency */
  double minimum_frequency;    /* TaylorF2 waveform argument (Hz) */
  const double *frequency;     /* [n_bins] frequency_array, host */
  const gwl_detector *detectors;
} gwl_analysis_desc;

typedef struct gwl_analysis gwl_analysis;

/* Create a device-resident analysis (base.py:150-229 minus marginalisation
 * set-up).  Copies and derives every table; the caller's arrays may be freed
 * on return. */
int gwl_analysis_create(const gwl_analysis_desc *desc, gwl_analysis **out);
int gwl_analysis_destroy(gwl_analysis *a);

/* Bytes of device memory the analysis holds (tables, not per-batch work space). */
int gwl_analysis_resident_bytes(const gwl_analysis *a, size_t *bytes);

/* noise_log_likelihood(): -sum_det |<d|d>| / 2 over masked bins (base.py:402-417). */
int gwl_noise_log_likelihood(gwl_analysis *a, double *out);

/* Time marginalisation (base.py:183-195, 325-330, 794-820, 1027-1035).
 * The geocent_time prior must be Uniform(t_min, t_max); jitter != 0 shifts
 * the time grid by each point's GWL_P_TIME_JITTER.  Requires the analysis
 * grid to have an even number of FFT points (n_bins - 1). */
int gwl_set_time_marginalization(gwl_analysis *a, int enable, int jitter, double t_min, double t_max);

/* A geocent_time prior other than Uniform for time marginalisation: the
 * reference weights each time sample t_j (jittered) by
 * priors['geocent_time'].prob(t_j) * delta_tc (bilby/gw/likelihood/base.py:
 * 794-820).  `density` holds that density on the n nodes t0 + g h, with h a
 * power of two (seconds) and t0 a multiple of h, so that every node time is
 * exact in float64; the kernels interpolate it with four nodes (one-sided at
 * the ends).  n = 0 returns to the Uniform prior of [t_min, t_max]. */
int gwl_set_time_prior(gwl_analysis *a, const double *density, int64_t n, double t0, double h);

/* Phase marginalisation (base.py:202-205, 786-792): ln I0(|<d|h>|) - <h|h>/2. */
int gwl_set_phase_marginalization(gwl_analysis *a, int enable);

/* Distance marginalisation (base.py:207-223, 775-784, 879-934): the caller
 * passes the interpolating bicubic B-spline of the lookup table that
 * BoundedRectBivariateSpline builds (core/utils/calculus.py:221-262), as
 * knots tx[nx], ty[ny] and coefficients c[(nx-4)*(ny-4)] (row major over x),
 * its bounding box, and the reference distance.  Outside the box the
 * result is -inf. */
int gwl_set_distance_marginalization(gwl_analysis *a, int enable, const double *tx, int32_t nx,
                                     const double *ty, int32_t ny, const double *c,
                                     const double bbox[4], double reference_distance);

/* The bound r_max = d_ref / d_min (at least 1) on the slope E[d_ref / d] of
 * the distance-marginalised lnL in <d|h> (base.py:775-784): with distance
 * and without time marginalisation the mixed-precision kernels scale their
 * <d|h> error bounds by r_max and their <h|h> ones by r_max^2 / 2 before
 * comparing them with the refinement tolerance, so that |dlnL| stays below
 * it for every point.  Default 1. */
int gwl_set_distance_slope(gwl_analysis *a, double max_slope);

/* log_likelihood_ratio for B points.
 *   params: device pointer to a [GWL_NPARAM][B] float64 block (slot-major)
 *   out:    device pointer to B float64 results
 *   stream: cudaStream_t (NULL = legacy default stream)
 * Asynchronous on `stream`.  Work space is allocated on the first call for
 * a given B and reused. */
int gwl_eval_device(gwl_analysis *a, const double *params, int64_t B, int32_t precision,
                    double *out, void *stream);

/* Same, with host parameter and result buffers: copies the parameter block
 * in, evaluates and copies the results out, then synchronises. */
int gwl_eval_host(gwl_analysis *a, const double *params, int64_t B, int32_t precision, double *out);

/* Per-point inner products for B points (device pointers): d_inner_h
 * (interleaved complex, summed over detectors) and optimal_snr_squared,
 * i.e. the _CalculatedSNRs totals of base.py:109-148 before marginalisation. */
int gwl_inner_products_device(gwl_analysis *a, const double *params, int64_t B, int32_t precision,
                              double *d_inner_h, double *h_inner_h, void *stream);

/* The time series of <d|h> that time marginalisation sums over, for B points
 * (device pointers, float64): series[b] is the length-L transform
 * 4/T FFT(h conj(d) / S)[j], j < L = n_frequencies - 1, summed over
 * detectors, interleaved complex ([B][2L] doubles), i.e. the
 * d_inner_h_array of base.py:325-330; h_inner_h[b] = <h|h>.  Needs time
 * marginalisation enabled.  With relative binning the transform is of the
 * rebuilt piecewise-linear waveform (relative.py:410-418), with multi-banding
 * of the scattered banded strain times the linear coefficients, length
 * Nbs[-1] / 2 (multiband.py:792-800); with ROQ the five-sample
 * interpolation at each sample of the marginalisation grid, length n_times
 * (roq.py:535-541, 604-651).  Asynchronous on `stream`. */
int gwl_time_series_device(gwl_analysis *a, const double *params, int64_t B, double *series, double *h_inner_h,
                           void *stream);

/* Source polarisations {plus, cross} of one parameter point on a frequency
 * grid (host in, host out, float64): source.py:1153-1209 for the
 * sine-Gaussian; the TaylorF2 model for GWL_MODEL_TAYLORF2.  `params` is one
 * [GWL_NPARAM] vector.  plus / cross are [2*n] interleaved complex. */
int gwl_source_polarizations(int32_t model, const double *frequency, int64_t n, const double *params,
                             double minimum_frequency, double *plus, double *cross);

/* Detector response of given polarisations (interferometer.py:303-368 with
 * identity calibration), host in / host out, float64. */
int gwl_detector_response(const gwl_detector *det, const double *frequency, int64_t n,
                          const double *plus, const double *cross, const double *params,
                          double *response);

/* The distance-marginalisation lookup table of base.py:994-1018 (host in /
 * host out, float64, built on the GPU): for the n-point distance grid with
 * prior density `prior`, reference distance `ref_dist` and the reference
 * axes of base.py:899-914 (n_dh <d|h> values, n_hh <h|h> values),
 *   table[i][j] = logsumexp_k(dh'_jk - hh_i s_k^2 / 2, b = prior_k dd) - log_norm,
 * s_k = ref_dist / d_k, dh'_jk = dh_j s_k (or ln I0(|dh_j s_k|) with phase
 * marginalisation).  `table` is [n_hh][n_dh] row major. */
int gwl_distance_lookup_table(const double *distance, const double *prior, int32_t n, double ref_dist,
                              const double *dh_axis, int32_t n_dh, const double *hh_axis, int32_t n_hh,
                              int phase_marginalization, double *table);

/* Evaluate host+device float64 helpers on the host (ln I0 of x, or the
 * bicubic spline): a test hook that needs no GPU.  what = 0: out[i] =
 * ln_i0(x[i]); what = 1: out[i] = spline(x[i], y[i]) with the knots and
 * coefficients passed as in gwl_set_distance_marginalization. */
int gwl_host_math(int what, const double *x, const double *y, int64_t n, const double *tx, int32_t nx,
                  const double *ty, int32_t ny, const double *c, const double bbox[4], double *out);

/* ---- several analyses in one launch --------------------------------------
 * A batcher evaluates, in one launch sequence, batches of points that belong
 * to different analyses (configurations of uneven duration, sampling rate
 * and detector count): a persistent kernel per detector count pulls work
 * units (analysis, 128-point tile, group of chunks) from an atomic counter.
 * With graphs enabled, the launch sequence of each batch shape (analyses and
 * point counts) is captured once in a CUDA graph and replayed.  Mixed
 * precision TaylorF2 analyses without time marginalisation take the fused
 * path; any other item is evaluated by its own launch sequence.  A batcher
 * holds its own work space, so one batcher serves one stream at a time.
 * This extends base.py:419-477 to many analyses at once; it has no single
 * counterpart in the reference, whose likelihood evaluates one point of one
 * analysis per call. */
typedef struct gwl_batcher gwl_batcher;

typedef struct {
  gwl_analysis *analysis;
  const double *params;   /* device [GWL_NPARAM][B] */
  int64_t B;
  double *out;            /* device [B] */
} gwl_batch_item;

int gwl_batcher_create(gwl_batcher **out);
int gwl_batcher_destroy(gwl_batcher *b);
int gwl_batcher_use_graphs(gwl_batcher *b, int enable);
int gwl_batcher_eval(gwl_batcher *b, const gwl_batch_item *items, int32_t n, int32_t precision, void *stream);
/* Reads and clears the batcher's device status word (non-zero: a bounded wait gave up). */
int gwl_batcher_status(gwl_batcher *b, int *device_status);

/* Zero-copy host staging: gwl_host_buffers returns the analysis's pinned
 * parameter block [GWL_NPARAM][B] and result buffer [B] (valid until a
 * larger batch, or a first gwl_time_series_device call on a relative-binning
 * or multi-banding analysis, reallocates them); the caller fills the block and calls
 * gwl_eval_host_staged, which runs gwl_eval_host without the two host
 * copies and leaves the lnL ratios in the result buffer.  Same results as
 * gwl_eval_host (no counterpart in the reference). */
int gwl_host_buffers(gwl_analysis *a, int64_t B, double **params, double **out);
int gwl_eval_host_staged(gwl_analysis *a, int64_t B, int32_t precision);

/* log_likelihood_ratio for B points without allocating device memory, for
 * callers that cannot let a library call cudaMalloc (an application that
 * reserves the GPU's memory for its own pool, or a latency-critical loop
 * that must not pay cudaMalloc's device-wide synchronisation).  It has no
 * counterpart in the reference.  Mixed-precision TaylorF2 analyses without
 * time marginalisation only (GWL_ERR_UNSUPPORTED otherwise).  params / out
 * are device pointers as for gwl_eval_device; asynchronous on `stream`; the
 * device status word is not read back (gwl_noalloc_status does).  The work space is a static 32 MiB
 * device buffer shared by all calls: B is limited to what fits (about 1,800
 * points for 128 s at 4096 Hz with 3 detectors, about 40,000 for 8 s at
 * 2048 Hz with 2 detectors); larger B returns GWL_ERR_ARGUMENT.  The first
 * call on a device looks up the buffer's address -- make it before any
 * stream capture.  Calls that overlap on the GPU race on the buffer. */
int gwl_eval_device_noalloc(gwl_analysis *a, const double *params, int64_t B, double *out, void *stream);

/* The status word of gwl_eval_device_noalloc's kernels on the current
 * device: waits for `stream`, writes the word to *device_status (0 = ok,
 * 1 = a bounded bulk-copy wait gave up, 2 = a point's ordering key out of
 * range) and clears it.  Returns GWL_OK for 0, GWL_ERR_TIMEOUT for 1 and
 * GWL_ERR_ARGUMENT for 2.  It allocates nothing.  No counterpart in the
 * reference. */
int gwl_noalloc_status(void *stream, int *device_status);

/* Measurement hooks: with profiling enabled, each evaluation records CUDA
 * events on its stream around its dominant kernel (the fused likelihood or
 * time-marginalisation kernel); gwl_profile_last_kernel_ms waits for the
 * last one and returns its duration in milliseconds. */
int gwl_set_profiling(gwl_analysis *a, int enable);
int gwl_profile_last_kernel_ms(gwl_analysis *a, float *ms);

/* Relative binning (replaces the per-evaluation part of
 * RelativeBinningGravitationalWaveTransient, bilby/gw/likelihood/relative.py:
 * calculate_snrs 365-402 through compute_waveform_ratio_per_interferometer;
 * the bins and summary data of setup_bins 178-230 and compute_summary_data
 * 319-363 are computed by the caller).  With it enabled, every evaluation of
 * this analysis evaluates the model at the n_edges bin edges (increasing
 * grid indices edge_index), forms the ratio to the fiducial response through
 * h0_inverse ([n_det][n_edges][2]: 1 / h0_d(f_e), re/im) and sums the per-bin
 * summary data ([n_det][n_edges - 1][6]: a0 re, a0 im, a1 re, a1 im, b0, b1)
 * in float64 for either precision.  Phase and distance marginalisation
 * apply; time marginalisation needs gwl_set_relative_binning_time_weights
 * as well (after each call of this function). */
int gwl_set_relative_binning(gwl_analysis *a, int enable, int32_t n_edges, const int64_t *edge_index,
                             const double *h0_inverse, const double *summary);

/* Relative binning with time marginalisation (relative.py:380-420): the
 * full-grid weights weights[d][k] = 4/T h0_d(f_k) conj(d_d(f_k)) / S_d(f_k)
 * ([n_det][n_bins][2], re/im; zero outside the frequency mask and outside
 * the first and last bin edges).  Each evaluation then rebuilds the
 * piecewise-linear waveform h0_d(f) (r0_b + r1_b (f - f_b)) on the grid,
 * transforms it against the data (float64, FFT length n_bins - 1) and
 * marginalises over time with <h|h> from the summary data. */
int gwl_set_relative_binning_time_weights(gwl_analysis *a, const double *weights);

/* Multi-banding (replaces MBGravitationalWaveTransient.calculate_snrs with
 * linear interpolation of <h|h>, bilby/gw/likelihood/multiband.py:741-819;
 * the bands and coefficients of setup_multibanding 317-640 are computed by
 * the caller).  With it enabled, every evaluation of this analysis evaluates
 * the model at the n_points banded frequencies, projects it on each detector
 * and forms <d|h> = conj(sum_k s_k L_k) and <h|h> = sum_k |s_k|^2 Q_k with
 * linear ([n_det][n_points][2], complex) and quadratic ([n_det][n_points])
 * coefficients, in float64 for either precision.  The banded frequencies
 * come in n_bands runs: band b holds indices [band_start[b], band_start[b+1])
 * uniformly spaced by band_df[b] (1 / T^(b)).  Phase and distance
 * marginalisation apply; time marginalisation needs
 * gwl_set_multiband_time_marginalization as well (after each call of this
 * function). */
int gwl_set_multiband(gwl_analysis *a, int enable, int64_t n_points, const double *frequencies,
                      const double *linear, const double *quadratic, int32_t n_bands, const int64_t *band_start,
                      const double *band_df);

/* Multi-banding with time marginalisation (multiband.py:714-726, 792-800):
 * the banded strain times the linear coefficients is scattered to the
 * full-resolution indices k < n_fft (a power of two, Nbs[-1] / 2) and
 * transformed (float64); time sample j is start + j delta_tc (+ jitter).
 * index_start [n_fft + 1] and source [n_points] list, for each k, the banded
 * points scattered there in band order: a code c >= 0 is banded point c; a
 * code c < 0 is banded point -c - 1, which a later point of its band replaced
 * at that index (it enters <h|h> only).  antenna_time fixes the time of the
 * antenna patterns (the reference sets the interferometers' reference_time
 * to the middle of the geocent_time prior); the delays stay at geocent_time. */
int gwl_set_multiband_time_marginalization(gwl_analysis *a, int64_t n_fft, const int32_t *index_start,
                                           const int32_t *source, double delta_tc, double antenna_time);

/* Multi-banding with the IFFT-FFT <h|h> (replaces the linear_interpolation=
 * False branch of MBGravitationalWaveTransient.calculate_snrs,
 * bilby/gw/likelihood/multiband.py:760-779, set up by
 * _setup_quadratic_coefficients_ifft_fft 613-650).  Call after
 * gwl_set_multiband (whose quadratic coefficients then hold band 0's direct
 * weights (4/T) mask w / S and, for bands b >= 1, the even bins' weights
 * (4/That_b) w_k Re I_b[2 m_k], m_k = K_s + k - k_b).  Per band b >= 1 and
 * detector every evaluation transforms W = sqrt(w) s over M = m[b] samples
 * and adds scale[b] sum_j |Z_j|^2 Re I_b[2j + 1] (the odd bins) to <h|h>:
 * in float64, or with GWL_PRECISION_MIXED and TaylorF2 in float32 with an
 * error bound per point, the points over the refinement tolerance
 * recomputed in float64.  ks[b] and m[b] ([n_bands], m[0] = 0, m[b] a
 * power of two with 1 <= ks[b] and ks[b] + n_b - 1 < m[b] / 2), scale[b] =
 * 4 / That_b, sqrt_window [n_points] the square roots of the band windows,
 * odd_weights [n_det][sum over b >= 1 of m[b] / 2] (Re I_b[2j + 1], band
 * after band).  enable = 0 switches it off; a new gwl_set_multiband does too. */
int gwl_set_multiband_ifft_fft(gwl_analysis *a, int enable, const int32_t *ks, const int32_t *m, const double *scale,
                               const double *sqrt_window, const double *odd_weights);

/* NVTX ranges (no-ops unless a profiler is attached).  The library marks
 * its entry points (gwl_eval_device, gwl_eval_host with its h2d / launch /
 * readback steps, gwl_batcher_eval); a caller marks its own phases, e.g. a
 * server's admission, with these.  No counterpart in the reference. */
int gwl_trace_push(const char *name);
int gwl_trace_pop(void);

/* Reduced-order quadrature (replaces ROQGravitationalWaveTransient.
 * calculate_snrs for one linear and one quadratic basis without time
 * marginalisation, bilby/gw/likelihood/roq.py:467-602; the weights of
 * _set_weights 736-1007 are computed by the caller).  With it enabled, every
 * evaluation evaluates the model at the n_linear linear and n_quadratic
 * quadratic frequency nodes, projects it on each detector (antenna patterns
 * only: the time shift lives in the weights), contracts the linear part with
 * the weights of the five time samples around the detector's arrival time
 * (time sample k at (time_start_index + k) * time_step, k < n_time;
 * linear_weights [n_det][n_time][n_linear][2]) and interpolates them to the
 * arrival time (LIGO-T2100224); <h|h> = sum_j |h(G_j)|^2 w_j
 * (quadratic_weights [n_det][n_quadratic]).  float64 for either precision;
 * an arrival time within two samples of the grid's ends gives lnL = -inf, as
 * in the reference.  Time marginalisation needs
 * gwl_set_roq_time_marginalization as well. */
int gwl_set_roq(gwl_analysis *a, int enable, int32_t n_linear, const double *nodes_linear, int32_t n_quadratic,
                const double *nodes_quadratic, int64_t n_time, int64_t time_start_index, double time_step,
                const double *linear_weights, const double *quadratic_weights);

/* ROQ with time marginalisation (roq.py:320-331, 535-541, 604-651): the
 * marginalisation grid times[n_times] (absolute GPS, increasing; the
 * reference's tc_min + delta_tc / 2 + j delta_tc), the weight delta_tc of
 * each sample, and antenna_time, the time of the antenna patterns and of the
 * detector delays (the middle of the geocent_time prior).  Each evaluation
 * then contracts the linear weights of every row its detector times read
 * with conj(h) at the linear nodes, interpolates <d|h> at each time sample
 * from five rows (LIGO-T2100224), sums over detectors and marginalises
 * (float64), in chunks of time samples whose rows fit in shared memory.
 * Refused when the linear nodes alone do not fit.  gwl_set_roq resets it. */
int gwl_set_roq_time_marginalization(gwl_analysis *a, int64_t n_times, const double *times, double delta_tc,
                                     double antenna_time);

/* On-device prior rescaling and parameter conversion for the batch path
 * (replaces, for the supported priors, PriorDict.rescale, bilby/core/prior/
 * dict.py, with the inverse CDFs of bilby/core/prior/analytical.py,
 * interpolated.py and bilby/gw/prior.py, followed by the mass and
 * inclination conversions of convert_to_lal_binary_black_hole_parameters,
 * bilby/gw/conversion.py:182-283, 849-990).  A program of n entries maps
 * unit-cube samples ([n_columns][B], device) to the [GWL_NPARAM][B]
 * parameter block (device) in one launch; entries with column < 0 are
 * constants (DeltaFunction). */
enum {
  GWL_PRIOR_DELTA = 0,       /* p[0] = peak */
  GWL_PRIOR_UNIFORM = 1,     /* p = minimum, maximum */
  GWL_PRIOR_POWERLAW = 2,    /* p = alpha, minimum, maximum (alpha = -1: log-uniform) */
  GWL_PRIOR_SINE = 3,        /* p = minimum, maximum */
  GWL_PRIOR_COSINE = 4,      /* p = minimum, maximum */
  GWL_PRIOR_GAUSSIAN = 5,    /* p = mu, sigma */
  GWL_PRIOR_TRUNCATED_GAUSSIAN = 6, /* p = mu, sigma, minimum, normalisation */
  GWL_PRIOR_TABLE_LINEAR = 7,  /* linear interpolation of the inverse CDF: x = CDF grid, y = values */
  GWL_PRIOR_TABLE_BSPLINE = 8  /* cubic B-spline inverse CDF: x = knots, y = coefficients,
                                  p = value below / above the knot range, equal-mass folding flag, last x */
};
/* Conversion targets beyond the parameter slots. */
enum {
  GWL_T_CHIRP_MASS = 100,
  GWL_T_MASS_RATIO = 101,
  GWL_T_TOTAL_MASS = 102,
  GWL_T_COS_THETA_JN = 103,
  GWL_T_ZENITH = 104,        /* detector-pair frame (gwl_priors_set_frame) */
  GWL_T_AZIMUTH = 105,
  GWL_T_DETECTOR_TIME = 106  /* arrival time at the reference detector (gwl_priors_set_frame) */
};
typedef struct gwl_prior {
  int32_t kind;          /* GWL_PRIOR_* */
  int32_t target;        /* a GWL_P_* slot or a GWL_T_* conversion input */
  int32_t column;        /* unit-cube column, or -1 for a constant */
  int32_t table_n;       /* table length (GWL_PRIOR_TABLE_*) */
  double p[4];
  const double *table_x; /* host arrays, copied by gwl_priors_create */
  const double *table_y;
} gwl_prior;
typedef struct gwl_priors gwl_priors;
int gwl_priors_create(const gwl_prior *entries, int32_t n, gwl_priors **out);
int gwl_priors_destroy(gwl_priors *p);
/* unit: device [n_columns][B]; params: device [GWL_NPARAM][B] (slots without
 * an entry are left as they are) */
int gwl_priors_rescale(gwl_priors *p, const double *unit, int64_t B, double *params, void *stream);

/* Detector-frame sampling for the batch path (get_sky_frame_parameters,
 * bilby/gw/likelihood/base.py:1091-1137): with `rotation` (the 3x3 row-major
 * rotation of the detector-pair frame, bilby/gw/geometry.py rotation_matrix_
 * from_delta) the GWL_T_ZENITH / GWL_T_AZIMUTH values become ra / dec at
 * the sampled time (the reference detector's arrival time when one is
 * sampled, else geocent_time); with `vertex` (the reference detector's
 * vertex, m) the GWL_T_DETECTOR_TIME value becomes geocent_time =
 * t - time_delay_from_geocenter(vertex, ra, dec, t).  NULL clears either. */
int gwl_priors_set_frame(gwl_priors *p, const double *rotation, const double *vertex);

/* Autotuner (no counterpart in the reference, which has no launch shapes):
 * times the mixed-precision TaylorF2 launch sequence on the caller's B device
 * points for each split-K depth (chunks of 512 bins walked by one CTA; 2, 3,
 * 4, 6, 8, 12, 16), keeps the fastest for this analysis and returns it with
 * its time (the fastest of five runs after one untimed run).  Synchronous on `stream`.  The depth sets the order in
 * which a point's chunk sums are added, so results are bit-reproducible for a
 * fixed depth and move by float64 rounding only (~1e-16 relative) when it
 * changes.  Other models and time marginalisation have nothing to tune. */
int gwl_autotune(gwl_analysis *a, const double *params, int64_t B, void *stream, int32_t *chunks_per_group,
                 double *best_ms);
int gwl_get_chunks_per_group(gwl_analysis *a, int32_t *chunks_per_group);
int gwl_set_chunks_per_group(gwl_analysis *a, int32_t chunks_per_group);

/* Error control of the mixed-precision TaylorF2 result (no counterpart in the
 * reference, which evaluates in float64 only).  The prologue bounds each
 * point's |Delta lnL| from prefix sums of the data weights:
 * 1e-6 L2 + 1e-7 L1, with L2 the Euclidean norm of the per-bin terms
 * |<d|h>_k| over the point's band and L1 their sum over the bins where the
 * data are signal-dominated (whitened power above 10), the place where the
 * error of the hardware cosine adds up coherently.  Points whose bound
 * exceeds `tolerance` (default 5e-4) are ordered first and evaluated by an
 * accurate variant of the kernel (float-float cosine from a table, TwoSum
 * accumulation of every term); tolerance <= 0 turns this off.  The choice
 * depends only on the point and the analysis, so a point's result does not
 * depend on the batch it is evaluated in.  gwl_last_refined waits for
 * `stream` and returns how many points the last mixed evaluation of `a`
 * marked; gwl_batcher_last_refined the same for the batcher's last launch. */
int gwl_set_refinement(gwl_analysis *a, double tolerance);
int gwl_get_refinement(gwl_analysis *a, double *tolerance);
int gwl_last_refined(gwl_analysis *a, void *stream, int64_t *count);
int gwl_batcher_last_refined(gwl_batcher *b, void *stream, int64_t *count);

/* Diagnostics of the failure path (no counterpart in the reference).
 * gwl_selftest_bounded_wait runs one CTA that arms a bulk-copy barrier for
 * 16 bytes and issues no copy, so the kernels' bounded wait must give up
 * after `poll_limit` polls: it returns GWL_ERR_TIMEOUT with *device_status = 1
 * and *arrived = 0, nothing left in flight.  gwl_inject_device_status writes
 * `value` into an analysis's device status word, as a kernel whose wait gave
 * up would, so that the next host evaluation reports it (GWL_ERR_TIMEOUT)
 * and clears it. */
int gwl_selftest_bounded_wait(uint32_t poll_limit, void *stream, int *device_status, int *arrived);
int gwl_inject_device_status(gwl_analysis *a, int value);

/* Description of the last error on this thread ("" if none). */
const char *gwl_last_error(void);

/* Library version string. */
const char *gwl_version(void);

#ifdef __cplusplus
}
#endif

#endif /* GWLNL_H */
