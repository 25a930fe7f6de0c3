/*
 * spx.h — C ABI of the GB300 FFT-to-peaks path (spectrum_gb300).
 *
 * This is the drop-in boundary for DspSpectrum's FFT -> |X| -> peaks hot path.
 * Every entry point takes plain pointers and sizes, returns an spx_status and
 * never throws.  Device pointers are borrowed; nothing returned here is owned
 * by the caller unless the comment says so.  All work is ordered on the
 * context's CUDA stream (spx_set_stream); entry points that fill device
 * buffers return before the GPU finishes, exactly like the reference's
 * *ToGPU / *ToBuffer calls.
 *
 * Mapping to the reference (paths relative to the DspSpectrum project):
 *   spx_fft                -> FFTProcessorROCm::ProcessComplex / ProcessMagPhase /
 *                             ProcessMagnitudesToGPU
 *                             (include/spectrum/fft_processor_rocm.hpp:74-124;
 *                              src/fft_func/src/fft_processor_rocm.cpp:306-659)
 *   spx_magnitude          -> ComplexToMagPhaseROCm::ProcessMagnitudeToBuffer /
 *                             ProcessMagnitudeToGPU / ProcessMagnitude
 *                             (include/spectrum/complex_to_mag_phase_rocm.hpp:187-225;
 *                              src/fft_func/src/complex_to_mag_phase_rocm.cpp:322-410)
 *   spx_mag_phase          -> ComplexToMagPhaseROCm::Process / ProcessToGPU
 *                             (complex_to_mag_phase_rocm.hpp:115-168)
 *   spx_peaks_one_two      -> SpectrumProcessorROCm post kernels (ONE_PEAK / TWO_PEAKS)
 *                             (include/spectrum/kernels/fft_kernel_sources_rocm.hpp:122-519,
 *                              src/fft_func/src/spectrum_processor_rocm.cpp:1030-1122)
 *   spx_all_maxima         -> IAllMaximaPipeline::Execute
 *                             (include/spectrum/interface/i_all_maxima_pipeline.hpp:71-80,
 *                              src/fft_func/src/all_maxima_pipeline_rocm.cpp:258-472)
 *   spx_topk               -> (no reference counterpart: top-K of local maxima)
 *   spx_fft_peaks          -> ISpectrumProcessor::ProcessFromGPU / FindAllMaximaFromGPUPipeline
 *                             fused: one launch up to nfft 16384, FFT + maxima launch
 *                             above (include/spectrum/interface/i_spectrum_processor.hpp:95-129)
 */
#ifndef SPX_H_
#define SPX_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SPX_ABI_VERSION 1

/* Status codes.  The C++ facades map INVALID_ARG to std::invalid_argument and
 * every other non-zero code to std::runtime_error, as the reference throws
 * (e.g. src/fft_func/src/spectrum_processor_rocm.cpp:267-277, 467-471). */
typedef enum spx_status {
  SPX_OK = 0,
  SPX_ERR_INVALID_ARG = 1,   /* null pointer, size mismatch, unsupported size */
  SPX_ERR_CUDA = 2,          /* a CUDA runtime call or launch failed */
  SPX_ERR_OUT_OF_MEMORY = 3, /* device allocation failed ("doesn't fit") */
  SPX_ERR_UNSUPPORTED = 4,   /* valid request this build does not implement */
  SPX_ERR_TIMEOUT = 5,       /* a bounded device-side wait gave up */
  SPX_ERR_NO_DEVICE = 6      /* no CUDA device / wrong device ordinal */
} spx_status;

/* One spectral maximum, 32 bytes; identical layout to antenna_fft::MaxValue
 * (include/spectrum/types/spectrum_result_types.hpp:34-43).  phase is in
 * DEGREES, refined_frequency = (index + freq_offset) * fs / nFFT. */
typedef struct spx_max_value {
  uint32_t index;
  float real;
  float imag;
  float magnitude;
  float phase;
  float freq_offset;
  float refined_frequency;
  uint32_t pad;
} spx_max_value;

/* Window applied to the n_point input samples before zero padding.
 * NONE..BLACKMAN match fft_processor::WindowType
 * (include/spectrum/types/window_type.hpp:26-31) with the (n_point-1)
 * denominator of pad_data_windowed (fft_processor_kernels_rocm.hpp:84-115);
 * BLACKMAN_HARRIS (4-term, same denominator) has no reference counterpart. */
enum spx_window {
  SPX_WINDOW_NONE = 0,
  SPX_WINDOW_HANN = 1,
  SPX_WINDOW_HAMMING = 2,
  SPX_WINDOW_BLACKMAN = 3,
  SPX_WINDOW_BLACKMAN_HARRIS = 4
};

/* Output of spx_fft.  COMPLEX: complex64 [beams x nfft], unnormalised.
 * MAG: float |X|*scale.  MAG2: float |X|^2*scale.  MAGPHASE: interleaved
 * float2 {|X|, atan2(im,re) radians} (complex_to_mag_phase). */
enum spx_fft_out {
  SPX_OUT_COMPLEX = 0,
  SPX_OUT_MAG = 1,
  SPX_OUT_MAG2 = 2,
  SPX_OUT_MAGPHASE = 3
};

/* Sub-bin refinement written into freq_offset / refined_frequency. */
enum spx_refine {
  SPX_REFINE_NONE = 0,      /* delta = 0, f = k*fs/nFFT (compact_maxima) */
  SPX_REFINE_PARABOLIC = 1  /* 3-point parabola on |X| (post_kernel_one_peak) */
};

enum spx_peak_mode {
  SPX_PEAK_ONE = 0,  /* ONE_PEAK: 4 MaxValue per beam */
  SPX_PEAK_TWO = 1,  /* TWO_PEAKS: 8 MaxValue per beam */
  SPX_PEAK_ALL = 2,  /* all strict local maxima, compacted */
  SPX_PEAK_TOPK = 3  /* K largest strict local maxima, magnitude-descending */
};

/* Peak-search parameters shared by the peak entry points.
 *  search_start/search_end: ALL/TOPK bin window [start, end); 0 -> 1 and
 *    0 -> nfft/2, end >= nfft -> nfft-1 (spectrum_processor_rocm.cpp:703-705).
 *  search_range: ONE/TWO window; 0 -> nfft/4 (spectrum_processor_rocm.cpp:1137-1143);
 *    bins [0, range/2) and [nfft-range/2, nfft) are searched.
 *  max_per_beam: ALL: output capacity per beam is
 *    min((end-start)/2, max_per_beam) (all_maxima_pipeline_rocm.cpp:304-307);
 *    TOPK: K (1..32).
 *  thresh_sigma: ALL/TOPK: keep maxima with |X| > noise_median * f(thresh_sigma)
 *    (see spx_noise_threshold_factor); 0 disables the threshold (reference
 *    behaviour).
 *  refine: spx_refine. */
typedef struct spx_peak_params {
  uint32_t mode;
  uint32_t search_start;
  uint32_t search_end;
  uint32_t search_range;
  uint32_t max_per_beam;
  uint32_t refine;
  float sample_rate;
  float thresh_sigma;
} spx_peak_params;

typedef struct spx_ctx spx_ctx;

/* ---- context ------------------------------------------------------------ */
/* Replaces the reference's IBackend/GpuContext pair (device + stream). */
spx_status spx_create(int device, spx_ctx** out);
spx_status spx_destroy(spx_ctx* ctx);
/* stream: a cudaStream_t (NULL = legacy default stream). */
spx_status spx_set_stream(spx_ctx* ctx, void* stream);
void* spx_get_stream(const spx_ctx* ctx);
spx_status spx_synchronize(spx_ctx* ctx);
/* Message of the last failing call on ctx ("" if none).  Valid until the next call. */
const char* spx_last_error(const spx_ctx* ctx);
const char* spx_status_string(spx_status status);
int spx_abi_version(void);
/* Bytes of grow-on-demand device scratch ctx holds now (look-back words,
 * thresholds, intermediate spectra, exchange slots), for memory accounting;
 * 0 for a context no call has needed scratch on yet.  No reference
 * counterpart (the reference's BufferSet does not report its size). */
uint64_t spx_scratch_bytes(const spx_ctx* ctx);

/* Self-test of the bounded device-side waits (no reference counterpart).
 * Every spin-wait in this library's kernels (the look-back of the all-maxima
 * scan) gives up after 1 s, sets the context's error word and lets the kernel
 * finish; the next spx_synchronize returns SPX_ERR_TIMEOUT and clears it.
 * This call runs one such wait on a predecessor that never publishes, so it
 * takes about 1 s and returns SPX_ERR_TIMEOUT; the context stays usable. */
spx_status spx_selftest_wait_timeout(spx_ctx* ctx);
/* The same for the per-beam group barrier of the large fused transform
 * (nfft > 16384): one CTA waits for a second arrival that never comes;
 * about 1 s, SPX_ERR_TIMEOUT, the context stays usable. */
spx_status spx_selftest_group_wait_timeout(spx_ctx* ctx);

/* ---- sizes -------------------------------------------------------------- */
/* nextPow2(n) as the reference computes it (fft_processor_rocm.cpp:665-671); 0 -> 1. */
uint32_t spx_next_pow2(uint32_t n);
/* Smallest 2^a*3^b >= n (extension for beams of uneven length). */
uint32_t spx_next_smooth23(uint32_t n);
/* 1 if this build can transform nfft points; else 0.  2^a*3^b in
 * [2, 262144]: one pass (cluster of <= 16 CTAs); 2^19 and 2^20: two
 * launches, 2^21: three; 2^a*3^b above 2^21 up to 2^28 that split into two factors
 * <= 16384 (every power of two): four steps with transposes; any other
 * length up to 2^27: Bluestein's chirp-z transform.  The reference takes any
 * nextPow2(n_point) * repeat_count (fft_processor_rocm.cpp:673-677). */
int spx_fft_size_supported(uint32_t nfft);
/* Tuning for transforms of nfft points: points each thread holds per pass
 * (16: more resident warps; 32: more work per thread) and, above 16384
 * points, the preferred points per CTA of a beam's cluster (1024..16384;
 * 0 = default 16384: one CTA per SM; 8192 allows two).  No reference counterpart (hipFFT
 * chooses internally); set by the autotuner or by hand. */
spx_status spx_set_fft_tuning(spx_ctx* ctx, uint32_t nfft, uint32_t points_per_thread,
                              uint32_t points_per_cta);
/* Resolves the ALL_MAXIMA defaults and returns the per-beam output capacity. */
spx_status spx_all_maxima_capacity(uint32_t nfft, uint32_t search_start,
                                   uint32_t search_end, uint32_t max_per_beam,
                                   uint32_t* start_out, uint32_t* end_out,
                                   uint32_t* cap_out);
/* Threshold multiplier applied to the per-beam noise median for thresh_sigma s:
 * (sqrt(pi/2) + s*sqrt(2 - pi/2)) / sqrt(2 ln 2), i.e. mean + s*std of a
 * Rayleigh-distributed noise magnitude expressed through its median. */
float spx_noise_threshold_factor(float thresh_sigma);

/* ---- FFT ---------------------------------------------------------------- */
/* Batched forward C2C FFT with window and zero padding.
 *  d_in : complex64 [beams x n_point] (device)
 *  nfft : >= n_point, 2^a*3^b; samples n_point..nfft-1 are zero
 *  out_mode / scale: spx_fft_out; scale multiplies MAG and MAG2 (inv_n), ignored otherwise
 *  d_out: [beams x nfft] of complex64 / float / float / float2 */
spx_status spx_fft(spx_ctx* ctx, const void* d_in, uint32_t beams,
                   uint32_t n_point, uint32_t nfft, uint32_t window,
                   uint32_t out_mode, float scale, void* d_out);

/* Batched inverse C2C FFT with 1/nfft scaling, x[n] = (1/nfft) sum_k X[k]
 * exp(+2 pi i k n / nfft): the reference's CpuFFT::InverseC2C
 * (include/spectrum/utils/cpu_fft.hpp:96-118) on the GPU.  d_in / d_out:
 * complex64 [beams x nfft]; d_out may equal d_in. */
spx_status spx_ifft(spx_ctx* ctx, const void* d_in, uint32_t beams, uint32_t nfft, void* d_out);

/* Batched FFT of real samples (float [beams x n_point]) with window and zero
 * padding to nfft as spx_fft.  full = 0: nfft/2 + 1 bins per beam
 * (CpuFFT::ForwardR2C, cpu_fft.hpp:131-152); full = 1: nfft bins, the upper
 * half the conjugate mirror X[nfft - k] = conj(X[k]) (CpuFFT::ForwardR2C_Full,
 * cpu_fft.hpp:165-180).  d_out: complex64 [beams x (nfft/2 + 1 or nfft)]. */
spx_status spx_fft_r2c(spx_ctx* ctx, const float* d_in, uint32_t beams, uint32_t n_point,
                       uint32_t nfft, uint32_t window, int full, void* d_out);

/* ---- magnitude / phase -------------------------------------------------- */
/* d_out[i] = |d_in[i]| * inv_n (squared: |d_in[i]|^2 * inv_n), count complex64 elements. */
spx_status spx_magnitude(spx_ctx* ctx, const void* d_in, float* d_out,
                         uint64_t count, float inv_n, int squared);
/* d_out[i] = {|d_in[i]|, atan2(im, re)} (radians), interleaved float2. */
spx_status spx_mag_phase(spx_ctx* ctx, const void* d_in, void* d_out,
                         uint64_t count);

/* ---- peak search on a spectrum ------------------------------------------ */
/* ONE_PEAK / TWO_PEAKS on a complex spectrum [beams x nfft]; writes 4 or 8
 * MaxValue per beam to d_out (post_kernel_one_peak / post_kernel_two_peaks). */
spx_status spx_peaks_one_two(spx_ctx* ctx, const void* d_fft, uint32_t beams,
                             uint32_t nfft, uint32_t search_range,
                             float sample_rate, int two_peaks,
                             spx_max_value* d_out);

/* All local maxima: detect -> scan -> compact.
 *  d_mag: float |X| [beams x nfft], or NULL to compute |X| from d_fft
 *  d_fft: complex64 [beams x nfft] (re/im/phase of each maximum)
 *  d_out: [beams x cap] (cap from spx_all_maxima_capacity)
 *  d_counts: [beams], the UNTRUNCATED number of maxima per beam. */
spx_status spx_all_maxima(spx_ctx* ctx, const float* d_mag, const void* d_fft,
                          uint32_t beams, uint32_t nfft,
                          const spx_peak_params* params,
                          spx_max_value* d_out, uint32_t* d_counts);

/* Top-K strict local maxima in [start, end), ordered by |X| descending, ties
 * by lower bin; d_out [beams x K], d_counts [beams] = number written (<= K). */
spx_status spx_topk(spx_ctx* ctx, const float* d_mag, const void* d_fft,
                    uint32_t beams, uint32_t nfft,
                    const spx_peak_params* params, spx_max_value* d_out,
                    uint32_t* d_counts);

/* All local maxima without any device allocation.  No counterpart in the
 * reference: it exists for callers that must not call cudaMalloc while they
 * run (a real-time loop that reserves its memory at start-up, or a host
 * framework that owns all device memory through its own pool), which
 * spx_all_maxima cannot serve because it grows a scratch buffer on demand.
 * Same arguments, layouts and results as spx_all_maxima, except:
 *  - thresh_sigma must be 0 (SPX_ERR_INVALID_ARG otherwise);
 *  - beams * ceil((end - start) / 2048) must be <= 32768 (SPX_ERR_INVALID_ARG);
 *  - its scratch is one fixed 256 KiB device array inside the library, held
 *    by every GPU that loads the library until exit and shared by all calls:
 *    calls whose kernels overlap on the GPU race, so order them on one stream;
 *  - the first call on a device looks the array's address up (once, with that
 *    device current) and, under CUDA's lazy module loading, loads the modules
 *    of the array and of the search kernel, which can allocate device memory
 *    once: make it during set-up, before any stream capture.
 * ctx is only used for its stream and error reporting (spx_create allocates
 * its small state once, before the no-allocation phase). */
spx_status spx_all_maxima_noalloc(spx_ctx* ctx, const float* d_mag, const void* d_fft,
                                  uint32_t beams, uint32_t nfft,
                                  const spx_peak_params* params,
                                  spx_max_value* d_out, uint32_t* d_counts);

/* ---- fused: raw samples -> peaks ---------------------------------------- */
/* Window + zero-pad + FFT + |X| + peak search.  nfft <= 16384 (ALL, TOPK):
 * one launch, the spectrum never goes to device memory.  ALL with nfft >
 * 16384: the FFT writes only the search window's bins (device scratch), then
 * one maxima launch.  Other cases: spx_fft, then the peak function.
 * params->mode selects ONE/TWO/ALL/TOPK with the layouts of
 * spx_peaks_one_two / spx_all_maxima / spx_topk.  d_counts may be NULL for
 * ONE/TWO; d_out may be NULL for ALL when the capacity is 0. */
spx_status spx_fft_peaks(spx_ctx* ctx, const void* d_in, uint32_t beams,
                         uint32_t n_point, uint32_t nfft, uint32_t window,
                         const spx_peak_params* params, spx_max_value* d_out,
                         uint32_t* d_counts);

/* ---- fused, host buffers -------------------------------------------------
 * spx_fft_peaks from host memory to host memory: the reference's
 * ISpectrumProcessor::ProcessFromCPU / FindAllMaximaFromCPU with
 * OutputDestination::CPU (include/spectrum/interface/i_spectrum_processor.hpp:85-86,
 * 117-119; src/fft_func/src/spectrum_processor_rocm.cpp:444-500).  h_in holds
 * beams x n_point complex64; h_out receives beams x R MaxValue (R = 4 ONE,
 * 8 TWO, the spx_all_maxima_capacity for ALL, K for TOPK) and h_counts the
 * per-beam counts (ALL/TOPK; may be NULL for ONE/TWO; h_out may be NULL when
 * R is 0).  Page-locked,
 * device-mapped input (cudaHostAlloc; cudaHostRegister with mapping) of at
 * most 112 MiB is read by the kernel in place over the host link; larger or
 * pageable input goes through in ~16 MiB chunks whose upload overlaps the
 * previous chunk's transform and search.  Page-locked, mapped outputs are
 * written by the kernel in place; others are copied back (per chunk, on a
 * third stream, when chunked).  Returns after the results are in host
 * memory. */
spx_status spx_fft_peaks_host(spx_ctx* ctx, const void* h_in, uint32_t beams,
                              uint32_t n_point, uint32_t nfft, uint32_t window,
                              const spx_peak_params* params, spx_max_value* h_out,
                              uint32_t* h_counts);

/* ---- batches of uneven beams ---------------------------------------------
 * No reference counterpart (DspSpectrum transforms one nFFT per call; its
 * nearest piece is host batching, src/fft_func/src/spectrum_processor_rocm.cpp:289-304).
 * A batch fixes B beams with their own n_point and nfft (nffts NULL or 0 ->
 * spx_next_smooth23(n_point)), the window and TOPK peak parameters
 * (params->mode must be SPX_PEAK_TOPK, K <= 32, thresh_sigma 0).  Every nfft
 * must run as C x M with C <= 16 CTAs of M <= 16384 points: 2^19 points
 * and more (multi-launch transforms) return SPX_ERR_UNSUPPORTED; run them
 * through spx_fft_peaks.  Inputs are packed: beam i's samples start at
 * sum_{j<i} n_point[j] (complex64); outputs are [B x K] MaxValue and [B]
 * counts, each beam's list the bits spx_fft_peaks gives for that beam alone.
 * Device scratch is owned by the batch.  A batch's plan for an nfft (its
 * local size M, C = nfft / M) is the context's plan for that nfft: every
 * call on the context uses it.
 *  spx_batch_run           every beam's FFT in ONE launch (clusters of the
 *                          largest C), then one top-K launch
 *  spx_batch_run_per_size  the same kernel once per distinct nfft (the
 *                          per-size baseline; bit-identical results)
 *  spx_batch_capture/replay  record spx_batch_run for fixed pointers as a
 *                          CUDA graph on the context's (non-default) stream
 *  spx_batch_tune          every size at the largest local size <= points_per_cta
 *                          (points_per_thread must be 16)
 *  spx_batch_local_size / spx_batch_set_local_size  one size's plan
 *  spx_batch_cluster / spx_batch_set_cluster  CTAs per cluster of the single
 *                          launch: 0 = the largest C of the batch's beams, or
 *                          any size from that to 16 (several beams share a
 *                          cluster; how many clusters fit at once depends on
 *                          how the size divides the GPU's SM groups)
 *  spx_batch_autotune      per distinct nfft, times the whole batch on the
 *                          given buffers with each candidate local size of that
 *                          nfft and keeps the fastest (the current plan unless
 *                          another is faster by over 2 %), then each cluster
 *                          size from the largest C to 16 the same way;
 *                          *sizes_tuned = sizes with more than one candidate,
 *                          *sizes_changed = plans changed (the cluster size
 *                          counts as one)
 *  spx_batch_save_plans / spx_batch_load_plans  the plans as a JSON file
 *                          {"arch": "sm_XY", "plans": {"<nfft>": M, ...},
 *                          "cluster": N}; loading applies the entries valid
 *                          for the batch's sizes on a device of that
 *                          architecture */
typedef struct spx_batch spx_batch;
spx_status spx_batch_create(spx_ctx* ctx, uint32_t beams, const uint32_t* n_points,
                            const uint32_t* nffts, uint32_t window,
                            const spx_peak_params* params, spx_batch** out);
spx_status spx_batch_destroy(spx_batch* batch);
uint64_t spx_batch_input_samples(const spx_batch* batch);
spx_status spx_batch_run(spx_ctx* ctx, spx_batch* batch, const void* d_in,
                         spx_max_value* d_out, uint32_t* d_counts);
spx_status spx_batch_run_per_size(spx_ctx* ctx, spx_batch* batch, const void* d_in,
                                  spx_max_value* d_out, uint32_t* d_counts);
spx_status spx_batch_capture(spx_ctx* ctx, spx_batch* batch, const void* d_in,
                             spx_max_value* d_out, uint32_t* d_counts);
spx_status spx_batch_replay(spx_ctx* ctx, spx_batch* batch);
spx_status spx_batch_tune(spx_ctx* ctx, spx_batch* batch, uint32_t points_per_thread,
                          uint32_t points_per_cta);
uint32_t spx_batch_local_size(const spx_batch* batch, uint32_t nfft);
uint32_t spx_batch_cluster(const spx_batch* batch);
spx_status spx_batch_set_cluster(spx_ctx* ctx, spx_batch* batch, uint32_t cluster);
spx_status spx_batch_set_local_size(spx_ctx* ctx, spx_batch* batch, uint32_t nfft,
                                    uint32_t local_size);
spx_status spx_batch_autotune(spx_ctx* ctx, spx_batch* batch, const void* d_in,
                              spx_max_value* d_out, uint32_t* d_counts,
                              uint32_t* sizes_tuned, uint32_t* sizes_changed);
spx_status spx_batch_save_plans(spx_ctx* ctx, const spx_batch* batch, const char* path);
spx_status spx_batch_load_plans(spx_ctx* ctx, spx_batch* batch, const char* path,
                                uint32_t* applied);

/* ---- learned sub-bin refinement ------------------------------------------
 * No reference counterpart: it stands beside the 3-point parabola of
 * include/spectrum/kernels/fft_kernel_sources_rocm.hpp:228-239 (the parabola
 * stays the fallback).  A 10 -> 64 -> 64 -> 2 GELU network with BF16 weights
 * and FP32 accumulation maps the 5 bins around a peak (|X[k+d]|/|X[k]| and
 * the window-corrected phase of X[k+d] conj X[k], d = -2..2) to the tone's
 * offset from bin k (bins) and log(amplitude / |X[k]|).
 * Parameters: spx_mlp_param_count() floats, layout W1[64][10] b1[64]
 * W2[64][64] b2[64] W3[2][64] b3[2] (FP32 masters; products read the BF16
 * rounding of the weights; biases are FP32).
 *  spx_mlp_make_frames  single-tone Hann frames made on the GPU: per frame the
 *                       features [10], the target [2] from a 16x zero-padded
 *                       FFT of the same frame, the parabolic result [2] =
 *                       (bin k, parabola offset), valid [1] and optionally
 *                       the truth [2] = (frequency in cycles/sample, SNR dB)
 *  spx_mlp_forward      Y[rows][2] from X[rows][10]
 *  spx_mlp_gradients    gradient of the masked mean squared error (mask NULL
 *                       = every row) w.r.t. the parameters; *d_loss += loss
 *  spx_mlp_train_step   one Adam step (beta 0.9 / 0.999, eps 1e-8)
 *  spx_mlp_train        epochs over rows (a power of two) in minibatches,
 *                       cosine learning rate lr_max -> lr_min, per-epoch mean
 *                       loss into d_epoch_loss[epochs] (may be NULL)
 *  spx_mlp_refine       rewrites freq_offset / refined_frequency of the
 *                       [beams x K] peaks of a TOPK/ALL search with counts;
 *                       keeps the parabolic values when the network's offset
 *                       leaves the bin; d_amplitude [beams x K] (may be NULL)
 *                       receives |X[k]| exp(y1); d_used_mlp (may be NULL)
 *                       1 where the network was used.
 * Training-data generation and training allocate; forward/refine allocate
 * activations only when a larger row count is first seen. */
typedef struct spx_mlp spx_mlp;
uint32_t spx_mlp_param_count(void);
spx_status spx_mlp_create(spx_ctx* ctx, uint64_t seed, spx_mlp** out);
spx_status spx_mlp_destroy(spx_mlp* mlp);
spx_status spx_mlp_set_params(spx_ctx* ctx, spx_mlp* mlp, const float* host_params);
spx_status spx_mlp_get_params(spx_ctx* ctx, spx_mlp* mlp, float* host_params);
spx_status spx_mlp_make_frames(spx_ctx* ctx, uint64_t seed, uint32_t frame0, uint32_t frames,
                               uint32_t nfft, float snr_lo_db, float snr_hi_db, float* d_feat,
                               float* d_target, float* d_parabolic, uint32_t* d_valid,
                               float* d_truth);
spx_status spx_mlp_forward(spx_ctx* ctx, spx_mlp* mlp, const float* d_x, uint32_t rows,
                           float* d_y);
spx_status spx_mlp_gradients(spx_ctx* ctx, spx_mlp* mlp, const float* d_x, const float* d_t,
                             const uint32_t* d_mask, uint32_t rows, float* d_grad,
                             float* d_loss);
spx_status spx_mlp_train_step(spx_ctx* ctx, spx_mlp* mlp, const float* d_x, const float* d_t,
                              const uint32_t* d_mask, uint32_t rows, float lr, float* d_loss);
spx_status spx_mlp_train(spx_ctx* ctx, spx_mlp* mlp, const float* d_feat,
                         const float* d_target, const uint32_t* d_valid, uint32_t rows,
                         uint32_t batch, uint32_t epochs, float lr_max, float lr_min,
                         uint64_t seed, float* d_epoch_loss);
spx_status spx_mlp_refine(spx_ctx* ctx, spx_mlp* mlp, const void* d_fft, uint32_t beams,
                          uint32_t n_point, uint32_t nfft, float sample_rate, uint32_t K,
                          spx_max_value* d_peaks, const uint32_t* d_counts,
                          float* d_amplitude, uint32_t* d_used_mlp);
/* spx_fft_peaks (params->mode SPX_PEAK_TOPK, K <= 32) followed by
 * spx_mlp_refine on its peaks, with the same results bit for bit.  Where one
 * CTA holds a beam's spectrum and the network's 20 KB of weights fit in the
 * spectrum's shared memory (2^a 3^b nfft from about 2600 to 16384 points),
 * and the call is small (beams x nfft <= 2^21), this is ONE launch:
 * transform, top-K search and the network on each peak, the spectrum never
 * written to device memory; otherwise the three steps run (faster once many
 * CTAs queue: one launch holds each SM while it stages the weights).  No reference counterpart (the
 * reference refines with the parabola, fft_kernel_sources_rocm.hpp:228-239). */
spx_status spx_fft_peaks_mlp(spx_ctx* ctx, spx_mlp* mlp, const void* d_in, uint32_t beams,
                             uint32_t n_point, uint32_t nfft, uint32_t window,
                             const spx_peak_params* params, spx_max_value* d_out,
                             uint32_t* d_counts, float* d_amplitude, uint32_t* d_used_mlp);

#ifdef __cplusplus
}  /* extern "C" */
#endif

#endif  /* SPX_H_ */
