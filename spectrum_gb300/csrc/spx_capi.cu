// spx_capi.cu — the extern "C" boundary (include/spx.h): argument checks,
// reference defaults, context / scratch management and dispatch to the
// kernels.  No exception crosses this boundary; every entry point returns an
// spx_status and records a message retrievable with spx_last_error.
#include <cmath>
#include <cstring>
#include <new>
#include <string>

#include "fft_core.cuh"
#include "spx_internal.h"

namespace spx {

spx_status fail(spx_ctx* ctx, spx_status st, const std::string& msg) {
  if (ctx) ctx->last_error = msg;
  return st;
}

spx_status cuda_fail(spx_ctx* ctx, cudaError_t e, const char* what) {
  const spx_status st =
      (e == cudaErrorMemoryAllocation) ? SPX_ERR_OUT_OF_MEMORY : SPX_ERR_CUDA;
  return fail(ctx, st, std::string(what) + ": " + cudaGetErrorName(e) + " (" +
                           cudaGetErrorString(e) + ")");
}

spx_status get_scratch(spx_ctx* ctx, int slot, size_t bytes, void** out) {
  if (bytes == 0) bytes = 256;
  if (ctx->scratch_bytes[slot] < bytes) {
    if (ctx->d_scratch[slot]) {
      cudaFree(ctx->d_scratch[slot]);
      ctx->d_scratch[slot] = nullptr;
      ctx->scratch_bytes[slot] = 0;
    }
    size_t sz = bytes + bytes / 4;  // headroom so slowly growing sizes do not thrash
    cudaError_t e = cudaMalloc(&ctx->d_scratch[slot], sz);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return cuda_fail(ctx, e, "cudaMalloc(scratch)");
    }
    ctx->scratch_bytes[slot] = sz;
  }
  *out = ctx->d_scratch[slot];
  return SPX_OK;
}

// Resolves ALL / TOPK window defaults (spectrum_processor_rocm.cpp:703-705).
static void resolve_window(uint32_t nfft, uint32_t* start, uint32_t* end) {
  if (*start == 0) *start = 1;
  if (*end == 0) *end = nfft / 2;
  if (*end >= nfft) *end = nfft - 1;
}

static spx_status peak_common_checks(spx_ctx* ctx, const spx_peak_params* p, uint32_t nfft) {
  if (!p) return fail(ctx, SPX_ERR_INVALID_ARG, "params is null");
  if (nfft < 3) return fail(ctx, SPX_ERR_INVALID_ARG, "nfft must be >= 3 for a peak search");
  if (p->refine > SPX_REFINE_PARABOLIC)
    return fail(ctx, SPX_ERR_INVALID_ARG, "unknown refine mode " + std::to_string(p->refine));
  if (!(p->thresh_sigma >= 0.0f) || std::isinf(p->thresh_sigma))
    return fail(ctx, SPX_ERR_INVALID_ARG, "thresh_sigma must be finite and >= 0");
  return SPX_OK;
}

// Per-beam thresholds for thresh_sigma > 0 (else *d_thr = null).
static spx_status thresholds(spx_ctx* ctx, const float* d_mag, const float2* d_fft,
                             uint32_t beams, uint32_t nfft, uint32_t start, uint32_t end,
                             float sigma, const float** d_thr) {
  *d_thr = nullptr;
  if (sigma <= 0.0f) return SPX_OK;
  void* t = nullptr;
  spx_status st = get_scratch(ctx, kSlotThresh, (size_t)beams * sizeof(float), &t);
  if (st != SPX_OK) return st;
  st = launch_noise_threshold(ctx, d_mag, d_fft, beams, nfft, start, end,
                              spx_noise_threshold_factor(sigma), static_cast<float*>(t));
  if (st != SPX_OK) return st;
  *d_thr = static_cast<const float*>(t);
  return SPX_OK;
}

}  // namespace spx

using namespace spx;

extern "C" {

int spx_abi_version(void) { return SPX_ABI_VERSION; }

uint64_t spx_scratch_bytes(const spx_ctx* ctx) {
  if (!ctx) return 0;
  uint64_t n = 0;
  for (size_t b : ctx->scratch_bytes) n += b;
  return n;
}

const char* spx_status_string(spx_status s) {
  switch (s) {
    case SPX_OK: return "SPX_OK";
    case SPX_ERR_INVALID_ARG: return "SPX_ERR_INVALID_ARG";
    case SPX_ERR_CUDA: return "SPX_ERR_CUDA";
    case SPX_ERR_OUT_OF_MEMORY: return "SPX_ERR_OUT_OF_MEMORY";
    case SPX_ERR_UNSUPPORTED: return "SPX_ERR_UNSUPPORTED";
    case SPX_ERR_TIMEOUT: return "SPX_ERR_TIMEOUT";
    case SPX_ERR_NO_DEVICE: return "SPX_ERR_NO_DEVICE";
  }
  return "SPX_ERR_UNKNOWN";
}

spx_status spx_create(int device, spx_ctx** out) {
  if (!out) return SPX_ERR_INVALID_ARG;
  *out = nullptr;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
    cudaGetLastError();
    return SPX_ERR_NO_DEVICE;
  }
  if (device < 0 || device >= n) return SPX_ERR_NO_DEVICE;
  spx_ctx* ctx = new (std::nothrow) spx_ctx();
  if (!ctx) return SPX_ERR_OUT_OF_MEMORY;
  ctx->device = device;
  DeviceGuard g(device);
  if (!g.ok) {
    delete ctx;
    return SPX_ERR_NO_DEVICE;
  }
  cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, device);
  if (ctx->sm_count <= 0) ctx->sm_count = 1;
  cudaError_t e = cudaMalloc(&ctx->d_error, sizeof(uint32_t));
  if (e == cudaSuccess) e = cudaMemset(ctx->d_error, 0, sizeof(uint32_t));
  if (e != cudaSuccess) {
    cudaGetLastError();
    delete ctx;
    return e == cudaErrorMemoryAllocation ? SPX_ERR_OUT_OF_MEMORY : SPX_ERR_CUDA;
  }
  *out = ctx;
  return SPX_OK;
}

spx_status spx_destroy(spx_ctx* ctx) {
  if (!ctx) return SPX_OK;
  {
    DeviceGuard g(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    ctx->plans.clear();
    for (auto& kv : ctx->windows) cudaFree(kv.second);
    for (int i = 0; i < kSlots; ++i)
      if (ctx->d_scratch[i]) cudaFree(ctx->d_scratch[i]);
    if (ctx->d_error) cudaFree(ctx->d_error);
    if (ctx->copy_in) {
      cudaStreamSynchronize(ctx->copy_in);
      cudaStreamDestroy(ctx->copy_in);
    }
    if (ctx->copy_out) {
      cudaStreamSynchronize(ctx->copy_out);
      cudaStreamDestroy(ctx->copy_out);
    }
    if (ctx->d_stage) cudaFree(ctx->d_stage);
    for (cudaEvent_t e : ctx->events) cudaEventDestroy(e);
  }
  delete ctx;
  return SPX_OK;
}

spx_status spx_set_stream(spx_ctx* ctx, void* stream) {
  if (!ctx) return SPX_ERR_INVALID_ARG;
  ctx->stream = static_cast<cudaStream_t>(stream);
  return SPX_OK;
}

void* spx_get_stream(const spx_ctx* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

const char* spx_last_error(const spx_ctx* ctx) { return ctx ? ctx->last_error.c_str() : ""; }

spx_status spx_synchronize(spx_ctx* ctx) {
  if (!ctx) return SPX_ERR_INVALID_ARG;
  DeviceGuard g(ctx->device);
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaStreamSynchronize");
  uint32_t err = 0;
  e = cudaMemcpy(&err, ctx->d_error, sizeof(err), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "read device error word");
  if (err) {
    cudaMemset(ctx->d_error, 0, sizeof(uint32_t));
    return fail(ctx, SPX_ERR_TIMEOUT,
                "a bounded device-side wait expired (error bits " + std::to_string(err) + ")");
  }
  return SPX_OK;
}

spx_status spx_selftest_wait_timeout(spx_ctx* ctx) {
  if (!ctx) return SPX_ERR_INVALID_ARG;
  DeviceGuard g(ctx->device);
  void* st = nullptr;
  spx_status s = get_scratch(ctx, kSlotWork, 2 * sizeof(unsigned long long), &st);
  if (s != SPX_OK) return s;
  s = launch_lookback_timeout_probe(ctx, static_cast<unsigned long long*>(st));
  if (s != SPX_OK) return s;
  return spx_synchronize(ctx);
}

spx_status spx_selftest_group_wait_timeout(spx_ctx* ctx) {
  if (!ctx) return SPX_ERR_INVALID_ARG;
  DeviceGuard g(ctx->device);
  void* st = nullptr;
  spx_status s = get_scratch(ctx, kSlotWork, sizeof(uint32_t), &st);
  if (s != SPX_OK) return s;
  s = launch_group_timeout_probe(ctx, static_cast<uint32_t*>(st));
  if (s != SPX_OK) return s;
  return spx_synchronize(ctx);
}

uint32_t spx_next_pow2(uint32_t n) {
  if (n == 0) return 1;
  n--;
  n |= n >> 1;
  n |= n >> 2;
  n |= n >> 4;
  n |= n >> 8;
  n |= n >> 16;
  return n + 1;
}

uint32_t spx_next_smooth23(uint32_t n) {
  if (n <= 1) return 1;
  uint64_t best = UINT64_MAX;
  for (uint64_t p2 = 1; p2 < ((uint64_t)n << 1); p2 <<= 1) {
    uint64_t v = p2;
    while (v < n) v *= 3;
    if (v < best) best = v;
  }
  return best > 0xFFFFFFFFull ? 0u : (uint32_t)best;
}

int spx_fft_size_supported(uint32_t nfft) {
  FftGeom g;
  return (build_geom(nfft, &g) || big_size(nfft) || huge_size(nfft) || bluestein_size(nfft)) ? 1 : 0;
}

spx_status spx_set_fft_tuning(spx_ctx* ctx, uint32_t nfft, uint32_t points_per_thread,
                              uint32_t points_per_cta) {
  if (!ctx) return SPX_ERR_INVALID_ARG;
  if (points_per_cta == 0) points_per_cta = kPrefLocalCluster;
  FftGeom g;
  if (!build_geom(nfft, &g, points_per_thread, points_per_cta))
    return fail(ctx, SPX_ERR_INVALID_ARG,
                "spx_set_fft_tuning: unsupported (nfft, points_per_thread, points_per_cta) = (" +
                    std::to_string(nfft) + ", " + std::to_string(points_per_thread) + ", " +
                    std::to_string(points_per_cta) + ")");
  ctx->tuning[nfft] = {points_per_thread, points_per_cta};
  return SPX_OK;
}

spx_status spx_all_maxima_capacity(uint32_t nfft, uint32_t search_start, uint32_t search_end,
                                   uint32_t max_per_beam, uint32_t* start_out,
                                   uint32_t* end_out, uint32_t* cap_out) {
  if (nfft < 3) return SPX_ERR_INVALID_ARG;
  resolve_window(nfft, &search_start, &search_end);
  // Unsigned arithmetic as in all_maxima_pipeline_rocm.cpp:304-307.
  uint32_t half = (uint32_t)(search_end - search_start) / 2u;
  uint32_t cap = half < max_per_beam ? half : max_per_beam;
  if (start_out) *start_out = search_start;
  if (end_out) *end_out = search_end;
  if (cap_out) *cap_out = cap;
  return SPX_OK;
}

float spx_noise_threshold_factor(float thresh_sigma) {
  const double pi = 3.14159265358979323846;
  const double s = (double)thresh_sigma;
  return (float)((std::sqrt(pi / 2.0) + s * std::sqrt(2.0 - pi / 2.0)) /
                 std::sqrt(2.0 * std::log(2.0)));
}

spx_status spx_fft(spx_ctx* ctx, const void* d_in, uint32_t beams, uint32_t n_point,
                   uint32_t nfft, uint32_t window, uint32_t out_mode, float scale, void* d_out) {
  if (!ctx) return SPX_ERR_INVALID_ARG;
  if (beams == 0) return SPX_OK;
  if (!d_in || !d_out) return fail(ctx, SPX_ERR_INVALID_ARG, "spx_fft: null device pointer");
  if (n_point == 0) return fail(ctx, SPX_ERR_INVALID_ARG, "spx_fft: n_point must be > 0");
  if (nfft < n_point)
    return fail(ctx, SPX_ERR_INVALID_ARG, "spx_fft: nfft must be >= n_point");
  if (out_mode > SPX_OUT_MAGPHASE)
    return fail(ctx, SPX_ERR_INVALID_ARG, "spx_fft: unknown out_mode");
  DeviceGuard g(ctx->device);
  const FftPlan* plan = nullptr;
  spx_status st = get_plan(ctx, nfft, &plan);
  if (st != SPX_OK) return st;
  const float* win = nullptr;
  st = get_window(ctx, window, n_point, &win);
  if (st != SPX_OK) return st;
  return launch_fft_out(ctx, *plan, static_cast<const float2*>(d_in), beams, n_point, win,
                        out_mode, scale, d_out);
}

spx_status spx_ifft(spx_ctx* ctx, const void* d_in, uint32_t beams, uint32_t nfft, void* d_out) {
  if (!ctx) return SPX_ERR_INVALID_ARG;
  if (beams == 0) return SPX_OK;
  if (!d_in || !d_out) return fail(ctx, SPX_ERR_INVALID_ARG, "spx_ifft: null device pointer");
  if (nfft == 0) return fail(ctx, SPX_ERR_INVALID_ARG, "spx_ifft: nfft must be > 0");
  DeviceGuard g(ctx->device);
  const FftPlan* plan = nullptr;
  spx_status st = get_plan(ctx, nfft, &plan);
  if (st != SPX_OK) return st;
  // x[n] = FFT(X)[(nfft - n) mod nfft] / nfft: the forward transform with a
  // reversing, scaling epilogue
  return launch_fft_out(ctx, *plan, static_cast<const float2*>(d_in), beams, nfft, nullptr,
                        kOutComplexReversed, 1.0f / (float)nfft, d_out);
}

spx_status spx_fft_r2c(spx_ctx* ctx, const float* d_in, uint32_t beams, uint32_t n_point,
                       uint32_t nfft, uint32_t window, int full, void* d_out) {
  if (!ctx) return SPX_ERR_INVALID_ARG;
  if (beams == 0) return SPX_OK;
  if (!d_in || !d_out) return fail(ctx, SPX_ERR_INVALID_ARG, "spx_fft_r2c: null device pointer");
  if (n_point == 0 || nfft < n_point)
    return fail(ctx, SPX_ERR_INVALID_ARG, "spx_fft_r2c: need 0 < n_point <= nfft");
  DeviceGuard g(ctx->device);
  const FftPlan* plan = nullptr;
  spx_status st = get_plan(ctx, nfft, &plan);
  if (st != SPX_OK) return st;
  const float* win = nullptr;
  st = get_window(ctx, window, n_point, &win);
  if (st != SPX_OK) return st;
  void* wide = nullptr;
  st = get_scratch(ctx, kSlotSpectrum, (size_t)beams * n_point * sizeof(float2), &wide);
  if (st != SPX_OK) return st;
  st = launch_widen_real(ctx, d_in, static_cast<float2*>(wide), (uint64_t)beams * n_point);
  if (st != SPX_OK) return st;
  return launch_fft_out(ctx, *plan, static_cast<const float2*>(wide), beams, n_point, win,
                        full ? kOutR2CFull : kOutR2CHalf, 1.0f, d_out);
}

spx_status spx_magnitude(spx_ctx* ctx, const void* d_in, float* d_out, uint64_t count,
                         float inv_n, int squared) {
  if (!ctx) return SPX_ERR_INVALID_ARG;
  if (count == 0) return SPX_OK;
  if (!d_in || !d_out) return fail(ctx, SPX_ERR_INVALID_ARG, "spx_magnitude: null pointer");
  DeviceGuard g(ctx->device);
  return launch_magnitude(ctx, static_cast<const float2*>(d_in), d_out, count, inv_n, squared);
}

spx_status spx_mag_phase(spx_ctx* ctx, const void* d_in, void* d_out, uint64_t count) {
  if (!ctx) return SPX_ERR_INVALID_ARG;
  if (count == 0) return SPX_OK;
  if (!d_in || !d_out) return fail(ctx, SPX_ERR_INVALID_ARG, "spx_mag_phase: null pointer");
  DeviceGuard g(ctx->device);
  return launch_mag_phase(ctx, static_cast<const float2*>(d_in), static_cast<float2*>(d_out),
                          count);
}

spx_status spx_peaks_one_two(spx_ctx* ctx, const void* d_fft, uint32_t beams, uint32_t nfft,
                             uint32_t search_range, float sample_rate, int two_peaks,
                             spx_max_value* d_out) {
  if (!ctx) return SPX_ERR_INVALID_ARG;
  if (beams == 0) return SPX_OK;
  if (!d_fft || !d_out) return fail(ctx, SPX_ERR_INVALID_ARG, "spx_peaks_one_two: null pointer");
  if (nfft < 2) return fail(ctx, SPX_ERR_INVALID_ARG, "spx_peaks_one_two: nfft must be >= 2");
  if (search_range == 0) search_range = nfft / 4;
  if (search_range < 2 || search_range > nfft)
    return fail(ctx, SPX_ERR_INVALID_ARG,
                "spx_peaks_one_two: search_range must be in [2, nfft] (got " +
                    std::to_string(search_range) + ")");
  DeviceGuard g(ctx->device);
  return launch_one_two(ctx, static_cast<const float2*>(d_fft), beams, nfft, search_range,
                        sample_rate, two_peaks, d_out);
}

spx_status spx_all_maxima(spx_ctx* ctx, const float* d_mag, const void* d_fft, uint32_t beams,
                          uint32_t nfft, const spx_peak_params* params, spx_max_value* d_out,
                          uint32_t* d_counts) {
  if (!ctx) return SPX_ERR_INVALID_ARG;
  spx_status st = peak_common_checks(ctx, params, nfft);
  if (st != SPX_OK) return st;
  if (beams == 0) return SPX_OK;
  if (!d_fft || !d_counts)
    return fail(ctx, SPX_ERR_INVALID_ARG, "spx_all_maxima: fft_data and counts are required");
  uint32_t start = 0, end = 0, cap = 0;
  spx_all_maxima_capacity(nfft, params->search_start, params->search_end, params->max_per_beam,
                          &start, &end, &cap);
  if (cap > 0 && !d_out) return fail(ctx, SPX_ERR_INVALID_ARG, "spx_all_maxima: out is null");
  DeviceGuard g(ctx->device);
  if (!d_mag && (end > start ? end - start : 0u) <= kMaxClusterSpan) {
    // one launch: |X|, noise threshold, maxima and ranks (maxima_cluster_kernel)
    void* scratch = nullptr;
    st = get_scratch(ctx, kSlotWork, (size_t)beams * 8 * sizeof(uint32_t), &scratch);
    if (st != SPX_OK) return st;
    const float factor = params->thresh_sigma > 0.0f ? spx_noise_threshold_factor(params->thresh_sigma) : 0.0f;
    return launch_maxima_cluster(ctx, static_cast<const float2*>(d_fft), 1, nfft, beams, nfft, start, end, cap,
                                 params->sample_rate, params->refine, factor,
                                 static_cast<uint32_t*>(scratch), d_out, d_counts);
  }
  const float* thr = nullptr;
  st = thresholds(ctx, d_mag, static_cast<const float2*>(d_fft), beams, nfft, start, end,
                  params->thresh_sigma, &thr);
  if (st != SPX_OK) return st;
  return launch_all_maxima(ctx, d_mag, static_cast<const float2*>(d_fft), beams, nfft, start,
                           end, cap, params->sample_rate, params->refine, thr, d_out, d_counts);
}

spx_status spx_topk(spx_ctx* ctx, const float* d_mag, const void* d_fft, uint32_t beams,
                    uint32_t nfft, const spx_peak_params* params, spx_max_value* d_out,
                    uint32_t* d_counts) {
  if (!ctx) return SPX_ERR_INVALID_ARG;
  spx_status st = peak_common_checks(ctx, params, nfft);
  if (st != SPX_OK) return st;
  const uint32_t K = params->max_per_beam;
  if (K < 1 || K > 32) return fail(ctx, SPX_ERR_INVALID_ARG, "spx_topk: K must be in [1, 32]");
  if (beams == 0) return SPX_OK;
  if (!d_fft || !d_out || !d_counts)
    return fail(ctx, SPX_ERR_INVALID_ARG, "spx_topk: null pointer");
  uint32_t start = params->search_start, end = params->search_end;
  resolve_window(nfft, &start, &end);
  DeviceGuard g(ctx->device);
  const float* thr = nullptr;
  st = thresholds(ctx, d_mag, static_cast<const float2*>(d_fft), beams, nfft, start, end,
                  params->thresh_sigma, &thr);
  if (st != SPX_OK) return st;
  return launch_topk(ctx, d_mag, static_cast<const float2*>(d_fft), beams, nfft, start, end, K,
                     params->sample_rate, params->refine, thr, d_out, d_counts);
}

spx_status spx_fft_peaks_mlp(spx_ctx* ctx, spx_mlp* mlp, const void* d_in, uint32_t beams, uint32_t n_point,
                             uint32_t nfft, uint32_t window, const spx_peak_params* params, spx_max_value* d_out,
                             uint32_t* d_counts, float* d_amplitude, uint32_t* d_used_mlp) {
  if (!ctx || !mlp) return SPX_ERR_INVALID_ARG;
  if (!params) return fail(ctx, SPX_ERR_INVALID_ARG, "params is null");
  if (params->mode != SPX_PEAK_TOPK)
    return fail(ctx, SPX_ERR_INVALID_ARG, "spx_fft_peaks_mlp: the learned refinement takes SPX_PEAK_TOPK");
  if (params->max_per_beam < 1 || params->max_per_beam > 32)
    return fail(ctx, SPX_ERR_INVALID_ARG, "spx_fft_peaks_mlp: K must be in [1, 32]");
  if (beams == 0) return SPX_OK;
  if (!d_in || !d_out || !d_counts) return fail(ctx, SPX_ERR_INVALID_ARG, "spx_fft_peaks_mlp: null device pointer");
  if (n_point == 0 || nfft < n_point)
    return fail(ctx, SPX_ERR_INVALID_ARG, "spx_fft_peaks_mlp: need 0 < n_point <= nfft");
  const void* pb = nullptr;
  const float* pw = nullptr;
  int mdev = 0;
  mlp_device_params(mlp, &pb, &pw, &mdev);
  if (mdev != ctx->device) return fail(ctx, SPX_ERR_INVALID_ARG, "spx_fft_peaks_mlp: the network is on another device");
  spx_status st = peak_common_checks(ctx, params, nfft);
  if (st != SPX_OK) return st;
  if (nfft < 5) return fail(ctx, SPX_ERR_INVALID_ARG, "spx_fft_peaks_mlp: need nfft >= 5");
  DeviceGuard g(ctx->device);
  const FftPlan* plan = nullptr;
  st = get_plan(ctx, nfft, &plan);
  if (st != SPX_OK) return st;
  const uint32_t K = params->max_per_beam;
  // One launch while the call is small (at most 2^21 points): each CTA then
  // also stages the network's weights and refines its peaks with one warp,
  // which pays while launch latency dominates; measured on GB300, 4096 x 8192
  // top-1 took 0.295 ms in one launch against 0.246 ms in three.
  const bool one_launch_pays = (uint64_t)beams * nfft <= (1ull << 21);
  if (!plan->big && !plan->bluestein && !plan->huge && one_launch_pays && fused_mlp_supported(plan->g, K)) {
    uint32_t start = params->search_start, end = params->search_end;
    resolve_window(nfft, &start, &end);
    const float* win = nullptr;
    st = get_window(ctx, window, n_point, &win);
    if (st != SPX_OK) return st;
    const MlpRefineArgs m{pb, pw, d_amplitude, d_used_mlp};
    const bool thr = params->thresh_sigma > 0.0f;
    return launch_fft_peaks(ctx, *plan, static_cast<const float2*>(d_in), beams, n_point, win, SPX_PEAK_TOPK,
                            start, end, K, params->sample_rate, params->refine,
                            thr ? spx_noise_threshold_factor(params->thresh_sigma) : 0.0f, d_out, d_counts, &m);
  }
  // other sizes: the spectrum in device memory, the search, then the refinement
  void* spec = nullptr;
  st = get_scratch(ctx, kSlotSpectrum, (size_t)beams * nfft * sizeof(float2), &spec);
  if (st != SPX_OK) return st;
  st = spx_fft(ctx, d_in, beams, n_point, nfft, window, SPX_OUT_COMPLEX, 1.0f, spec);
  if (st == SPX_OK) st = spx_topk(ctx, nullptr, spec, beams, nfft, params, d_out, d_counts);
  if (st != SPX_OK) return st;
  return spx_mlp_refine(ctx, mlp, spec, beams, n_point, nfft, params->sample_rate, K, d_out, d_counts,
                        d_amplitude, d_used_mlp);
}

spx_status spx_fft_peaks(spx_ctx* ctx, const void* d_in, uint32_t beams, uint32_t n_point,
                         uint32_t nfft, uint32_t window, const spx_peak_params* params,
                         spx_max_value* d_out, uint32_t* d_counts) {
  if (!ctx) return SPX_ERR_INVALID_ARG;
  if (!params) return fail(ctx, SPX_ERR_INVALID_ARG, "params is null");
  if (params->mode > SPX_PEAK_TOPK)
    return fail(ctx, SPX_ERR_INVALID_ARG, "unknown peak mode " + std::to_string(params->mode));
  if (beams == 0) return SPX_OK;
  if (!d_in) return fail(ctx, SPX_ERR_INVALID_ARG, "spx_fft_peaks: null device pointer");
  if (n_point == 0 || nfft < n_point)
    return fail(ctx, SPX_ERR_INVALID_ARG, "spx_fft_peaks: need 0 < n_point <= nfft");
  // the output may be null only for ALL with a zero capacity (nothing is written, as in spx_all_maxima)
  if (!d_out) {
    uint32_t s0 = 0, e0 = 0, cap0 = 1;
    if (params->mode == SPX_PEAK_ALL)
      spx_all_maxima_capacity(nfft, params->search_start, params->search_end, params->max_per_beam, &s0, &e0, &cap0);
    if (cap0 > 0) return fail(ctx, SPX_ERR_INVALID_ARG, "spx_fft_peaks: null device pointer");
  }
  DeviceGuard g(ctx->device);
  const FftPlan* plan = nullptr;
  spx_status st = get_plan(ctx, nfft, &plan);
  if (st != SPX_OK) return st;
  // Fused path: ALL maxima and TOP-K in one launch for C == 1 (the spectrum
  // stays on chip); ALL maxima for C > 1 as the beam-group (or cluster) FFT,
  // which writes only the window's bins, and the maxima cluster kernel.
  if (params->mode == SPX_PEAK_ALL || params->mode == SPX_PEAK_TOPK) {
    st = peak_common_checks(ctx, params, nfft);
    if (st != SPX_OK) return st;
    if (!d_counts) return fail(ctx, SPX_ERR_INVALID_ARG, "spx_fft_peaks: counts is null");
    const bool all = params->mode == SPX_PEAK_ALL;
    uint32_t start = params->search_start, end = params->search_end, cap = 0;
    if (all) {
      spx_all_maxima_capacity(nfft, start, end, params->max_per_beam, &start, &end, &cap);
    } else {
      if (params->max_per_beam < 1 || params->max_per_beam > 32)
        return fail(ctx, SPX_ERR_INVALID_ARG, "spx_fft_peaks: K must be in [1, 32]");
      resolve_window(nfft, &start, &end);
      cap = params->max_per_beam;
    }
    const bool thr = params->thresh_sigma > 0.0f;
    // nfft <= 16384 (one CTA per beam): the fused kernel keeps the spectrum
    // on chip, but its search phase holds the SM from the next beam's
    // transform, which pays only while the launch is short.  Measured on
    // GB300 (8 .. 4096 beams of 4096 .. 16384 points, top-1/8 and 6-sigma
    // all maxima), fused is faster for top-K at 4096 points or up to 2^23
    // points in all, and for all maxima up to 2^21 points in all; beyond, the
    // spectrum in device memory and a separate search kernel win (e.g. 4096
    // x 16384 top-8: 0.597 vs 0.463 ms).  Both give the same bits.
    const uint64_t pts = (uint64_t)beams * nfft;
    const bool single_cta_pays =
        plan->g.C > 1 || (all ? pts <= (1ull << 21) : (nfft <= 4096 || pts <= (1ull << 23)));
    if (!plan->big && !plan->bluestein && !plan->huge && single_cta_pays && fused_supported(plan->g, params->mode)) {
      const float* win = nullptr;
      st = get_window(ctx, window, n_point, &win);
      if (st != SPX_OK) return st;
      return launch_fft_peaks(ctx, *plan, static_cast<const float2*>(d_in), beams, n_point, win,
                              params->mode, start, end, cap, params->sample_rate, params->refine,
                              thr ? spx_noise_threshold_factor(params->thresh_sigma) : 0.0f,
                              d_out, d_counts);
    }
  }
  // Composed path: spectrum to device memory, then the peak kernels.
  void* spec = nullptr;
  st = get_scratch(ctx, kSlotSpectrum, (size_t)beams * nfft * sizeof(float2), &spec);
  if (st != SPX_OK) return st;
  st = spx_fft(ctx, d_in, beams, n_point, nfft, window, SPX_OUT_COMPLEX, 1.0f, spec);
  if (st != SPX_OK) return st;
  switch (params->mode) {
    case SPX_PEAK_ONE:
    case SPX_PEAK_TWO:
      return spx_peaks_one_two(ctx, spec, beams, nfft, params->search_range,
                               params->sample_rate, params->mode == SPX_PEAK_TWO, d_out);
    case SPX_PEAK_ALL:
      return spx_all_maxima(ctx, nullptr, spec, beams, nfft, params, d_out, d_counts);
    default:
      return spx_topk(ctx, nullptr, spec, beams, nfft, params, d_out, d_counts);
  }
}

}  // extern "C"
