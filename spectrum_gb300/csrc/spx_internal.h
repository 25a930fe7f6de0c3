// spx_internal.h — host-side state shared by the translation units of the
// spectrum_gb300 library (not installed; the public boundary is spx.h).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <map>
#include <memory>
#include <string>
#include <vector>

#include "spx.h"
#include "spx_geom.h"

namespace spx {

// Device-resident FFT plan for one nfft.
struct FftPlan {
  FftGeom g{};
  float2* d_tw_local = nullptr;  // M - 1 entries (>= 1 allocated)
  float2* d_tw_cross = nullptr;  // W_N^{n2}, M entries (big plans: W_N^{n2 k1} as [k1][n2], then W_Cb^e)
  bool big = false;              // three-launch transform (2^19, 2^20, 2^21 points)
  // Sizes without a direct plan: Bluestein's chirp-z transform through a
  // power-of-two transform of bm >= 2 nfft - 1 points (fft_bluestein.cu).
  bool bluestein = false;
  uint32_t bm = 0;
  const FftPlan* sub = nullptr;  // the bm-point plan (owned by the context)
  float2* d_chirp = nullptr;     // w[n] = exp(-i pi n^2 / nfft), n < nfft
  float2* d_bfft = nullptr;      // FFT_bm of the conjugate chirp, wrapped
  // Transforms of more than 2^21 points (fft_huge.cu): nfft = hn1 x hn2,
  // sub = the hn1-point plan, sub2 = the hn2-point plan, d_tw_cross = the
  // twiddle tables W_N^l (l < 2^hlshift), then W_N^{j 2^hlshift}.
  bool huge = false;
  uint32_t hn1 = 0, hn2 = 0, hlshift = 0;
  const FftPlan* sub2 = nullptr;
  ~FftPlan();
};

// Fills g for nfft with `ept` points per thread (16 or 32); returns false
// when nfft is not a supported single-pass size.
bool build_geom(uint32_t nfft, FftGeom* g, uint32_t ept = kEPTDefault,
                uint32_t pref_local = kPrefLocalCluster);
bool is_smooth23(uint32_t n);
// The local passes' twiddle table of geometry g (FP64-generated, FP32 stored):
// per pass, tw_rows(R) rows of W_{Ns R}^{r k}, or the two factors of a split
// radix-4 table (tw_split); g.twoff gives each pass's first entry.
void fill_local_twiddles(const FftGeom& g, float2* twl);


}  // namespace spx

struct spx_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  int sm_count = 0;
  std::string last_error;
  std::map<uint64_t, std::unique_ptr<spx::FftPlan>> plans;  // (ept, points/CTA, nfft)
  std::map<uint32_t, std::pair<uint32_t, uint32_t>> tuning;  // nfft -> (points/thread, points/CTA)
  std::map<uint64_t, float*> windows;  // (window << 32 | n_point) -> table
  // Grow-on-demand device scratch, one buffer per slot (see spx::Slot).
  void* d_scratch[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  size_t scratch_bytes[6] = {0, 0, 0, 0, 0, 0};
  uint32_t* d_error = nullptr;         // device error word (kErr* bits)
  uint32_t epoch = 0;                  // lookback status epoch
  // Host-buffer pipeline (spx_fft_peaks_host): copy streams, staging, events.
  cudaStream_t copy_in = nullptr, copy_out = nullptr;
  void* d_stage = nullptr;
  size_t stage_bytes = 0;
  std::vector<cudaEvent_t> events;
  // Set while a launch reads its samples from host memory (no L2 prefetch).
  bool input_on_host = false;
};

namespace spx {

// Records msg as the context's last error and returns st.
spx_status fail(spx_ctx* ctx, spx_status st, const std::string& msg);
// Maps a CUDA error to SPX_ERR_CUDA / SPX_ERR_OUT_OF_MEMORY with a message.
spx_status cuda_fail(spx_ctx* ctx, cudaError_t e, const char* what);

// Cached plan / window table (created on first use on the context's device).
spx_status get_plan(spx_ctx* ctx, uint32_t nfft, const FftPlan** out);
spx_status get_window(spx_ctx* ctx, uint32_t window, uint32_t n_point, const float** out);
// Scratch slots: buffers that must stay valid at the same time use different slots.
enum Slot : int {
  kSlotWork = 0,    // look-back status words, tickets, histograms
  kSlotThresh = 1,  // per-beam noise thresholds
  kSlotSpectrum = 2, // intermediate spectra of composed (non-fused) calls
  kSlotExchange = 3, // per-cluster exchange slots of the large-FFT kernels
  kSlotChirp = 4,    // the padded chirp-z sequences of Bluestein transforms
  kSlotHuge = 5      // the two transposed copies of a transform of more than 2^21 points
};
constexpr int kSlots = 6;
// Ensures at least `bytes` in `slot`; returns its device pointer.  Growing a
// slot frees the old buffer (cudaFree waits for the device first).
spx_status get_scratch(spx_ctx* ctx, int slot, size_t bytes, void** out);

// Raises a kernel's dynamic shared-memory limit (and allows clusters of
// up to 16) once per (device, kernel).
cudaError_t configure_kernel(const void* kernel, size_t max_smem);

// Largest transform without a direct plan (Bluestein, through a power of
// two of at most 2^28 points).
constexpr uint32_t kMaxBluestein = 1u << 27;
// Largest transform of the four-step path of fft_huge.cu (16384 x 16384).
constexpr uint32_t kMaxHuge = 1u << 28;
bool bluestein_size(uint32_t nfft);
spx_status build_bluestein_plan(spx_ctx* ctx, uint32_t nfft, FftPlan* plan);
spx_status launch_fft_bluestein(spx_ctx* ctx, const FftPlan& plan, const float2* d_in, uint32_t beams,
                                uint32_t n_point, const float* d_win, uint32_t out_mode, float scale,
                                void* d_out);
// Three-launch transforms of 2^19, 2^20 and 2^21 points (fft_big.cu).
bool big_size(uint32_t nfft);
spx_status build_big_plan(spx_ctx* ctx, uint32_t nfft, FftPlan* plan);
spx_status launch_fft_big(spx_ctx* ctx, const FftPlan& plan, const float2* d_in, uint32_t beams,
                          uint32_t n_point, const float* d_win, uint32_t out_mode, float scale,
                          void* d_out);

// Transforms of more than 2^21 points: N1 x N2, both 2^a 3^b <= 16384 (fft_huge.cu).
bool huge_size(uint32_t nfft);
spx_status build_huge_plan(spx_ctx* ctx, uint32_t nfft, FftPlan* plan);
spx_status launch_fft_huge(spx_ctx* ctx, const FftPlan& plan, const float2* d_in, uint32_t beams,
                           uint32_t n_point, const float* d_win, uint32_t out_mode, float scale,
                           void* d_out);

// Fused FFT + peak search (fft_peaks.cu).
bool fused_supported(const FftGeom& g, uint32_t mode);
// The learned refinement inside the single-CTA top-K launch: the network's
// BF16 products and FP32 biases, and the amplitude / used outputs (may be null).
struct MlpRefineArgs {
  const void* pb;
  const float* p;
  float* amp;
  uint32_t* used;
};
// Whether geometry g's single-CTA kernel can refine K peaks per beam with the
// network in its shared memory (C == 1 and room for the weights).
bool fused_mlp_supported(const FftGeom& g, uint32_t K);
spx_status launch_fft_peaks(spx_ctx* ctx, const FftPlan& plan, const float2* d_in,
                            uint32_t beams, uint32_t n_point, const float* d_win,
                            uint32_t mode, uint32_t start, uint32_t end, uint32_t cap_or_k,
                            float fs, uint32_t refine, float factor, spx_max_value* d_out,
                            uint32_t* d_counts, const MlpRefineArgs* mlp = nullptr);
// The device weights of a network (mlp.cu).
void mlp_device_params(const spx_mlp* mlp, const void** pb, const float** p, int* device);
// Output of C spectrum rows per beam (rows[beam][k1][q] = X[k1 + C*q], the
// exchange-slot layout) to bin order in any output mode (fft_kernels.cu).
spx_status launch_rows_transpose(spx_ctx* ctx, const FftGeom& g, const float2* rows, uint32_t beams,
                                 void* d_out, uint32_t out_mode, float scale);
// Geometries the persistent beam-group kernels take (power-of-two local size
// M in {4096, 8192, 16384} with M/16 threads, C in {2, 4, 8, 16}).
bool group_geometry(const FftGeom& g);
// Self-test of the group barrier's bounded wait (one CTA, two arrivals expected).
spx_status launch_group_timeout_probe(spx_ctx* ctx, uint32_t* d_count);
// Longest search window maxima_cluster_kernel takes (8 CTAs x 32768 bins).
constexpr uint32_t kMaxClusterSpan = 8u * 32768u;
// All maxima of spectra whose bin k of beam b sits at
// d_spec[b*nfft + (k mod C1)*M1 + k div C1] (C1 = 1: natural order), with the
// noise threshold when factor > 0; d_ccount holds beams * 8 words of scratch.
spx_status launch_maxima_cluster(spx_ctx* ctx, const float2* d_spec, uint32_t C1, uint32_t M1,
                                 uint32_t beams, uint32_t nfft, uint32_t start, uint32_t end,
                                 uint32_t cap, float fs, uint32_t refine, float factor,
                                 uint32_t* d_ccount, spx_max_value* d_out, uint32_t* d_counts);

// Kernel launchers (fft_kernels.cu, peak_kernels.cu).
spx_status launch_fft_out(spx_ctx* ctx, const FftPlan& plan, const float2* d_in,
                          uint32_t beams, uint32_t n_point, const float* d_win,
                          uint32_t out_mode, float scale, void* d_out);
spx_status launch_magnitude(spx_ctx* ctx, const float2* d_in, float* d_out,
                            uint64_t count, float inv_n, int squared);
spx_status launch_mag_phase(spx_ctx* ctx, const float2* d_in, float2* d_out,
                            uint64_t count);
spx_status launch_one_two(spx_ctx* ctx, const float2* d_fft, uint32_t beams,
                          uint32_t nfft, uint32_t search_range, float fs,
                          int two_peaks, spx_max_value* d_out);
// All local maxima (detect + decoupled-lookback scan + compact); thr may be
// null (no threshold) or hold one threshold per beam.
spx_status launch_all_maxima(spx_ctx* ctx, const float* d_mag, const float2* d_fft,
                             uint32_t beams, uint32_t nfft, uint32_t start,
                             uint32_t end, uint32_t cap, float fs, uint32_t refine,
                             const float* d_thr, spx_max_value* d_out,
                             uint32_t* d_counts);
// Look-back tiles (thread blocks) of one all-maxima launch.
uint64_t all_maxima_tiles(uint32_t beams, uint32_t start, uint32_t end);
// launch_all_maxima without threshold, with caller-provided scratch (no allocation).
spx_status launch_all_maxima_in(spx_ctx* ctx, const float* d_mag, const float2* d_fft,
                                uint32_t beams, uint32_t nfft, uint32_t start, uint32_t end,
                                uint32_t cap, float fs, uint32_t refine, spx_max_value* d_out,
                                uint32_t* d_counts, void* scratch, size_t scratch_bytes);
spx_status launch_topk(spx_ctx* ctx, const float* d_mag, const float2* d_fft,
                       uint32_t beams, uint32_t nfft, uint32_t start, uint32_t end,
                       uint32_t k, float fs, uint32_t refine, const float* d_thr,
                       spx_max_value* d_out, uint32_t* d_counts);
// CTAs (or beams of geometry g) of a launch of `kernel` resident at once:
// the L2 prefetch distance of the FFT kernels.
uint32_t resident_ctas(const void* kernel, uint32_t threads, size_t smem, uint32_t cluster);
uint32_t resident_beams(const void* kernel, const FftGeom& g, size_t smem);
// Real samples widened to complex (imaginary part 0).
spx_status launch_widen_real(spx_ctx* ctx, const float* d_in, float2* d_out, uint64_t n);
// Launches one bounded look-back wait that cannot be satisfied (self-test of
// the timeout path); d_status: 2 words of scratch.
spx_status launch_lookback_timeout_probe(spx_ctx* ctx, unsigned long long* d_status);
// Per-beam noise threshold: median estimate of |X| over [start, end) times factor.
spx_status launch_noise_threshold(spx_ctx* ctx, const float* d_mag, const float2* d_fft,
                                  uint32_t beams, uint32_t nfft, uint32_t start,
                                  uint32_t end, float factor, float* d_thr);

// Makes ctx's device current for the duration of an entry point.
struct DeviceGuard {
  int prev = -1;
  bool ok = true;
  explicit DeviceGuard(int dev) {
    if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
    if (prev != dev) ok = cudaSetDevice(dev) == cudaSuccess;
  }
  ~DeviceGuard() {
    int cur = -1;
    if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
  }
};

}  // namespace spx
