// host_pipeline.cu — spx_fft_peaks_host: raw samples in host memory -> peaks
// in host memory, the path of SpectrumProcessorROCm::ProcessFromCPU /
// FindAllMaximaFromCPU (src/fft_func/src/spectrum_processor_rocm.cpp:444-500:
// upload, FFT, peak search, read back).
//
// The host link carries ~210 GB/s whichever engine drives it (copy engines
// on one or several streams, or a kernel reading page-locked memory), so the
// upload of the samples sets the floor and the question is how much of the
// transform and the search hides behind it.
//
// Page-locked input that the device can address (cudaHostAlloc, or
// cudaHostRegister with mapping) of at most kZeroCopyMaxBytes is read by the
// kernel in place over the host link: no pipeline fill or drain, but the
// maxima kernel of every beam runs after the last sample has arrived.
//
// Larger input, and pageable input, goes through in chunks of about
// kChunkBytes of samples on the copy-in stream (host -> device) and the
// context's stream (the fused spx_fft_peaks launch), so the upload of chunk
// i + 1 overlaps the transform and search of chunk i and only the last
// chunk's compute is exposed.  The peaks are written by the kernel straight
// into mapped output buffers; other output comes back per chunk on the
// copy-out stream.  Staging: three input slots (and, for copied-back output,
// two output slots) in one device buffer owned by the context.  Events order
// slot reuse:
//   copy-in of chunk i waits until chunk i - 3 was computed (its input slot);
//   compute of chunk i waits for its upload and for the read-back of chunk
//   i - 2 (its output slot).
// With pageable host memory the chunk copies are still correct but do not
// overlap.
//
// Measured on the all-maxima search of 65536-point beams (nFFT 131072):
// 128 beams (64 MiB) 0.415 ms in place vs 0.454 ms chunked; 256 beams
// (128 MiB) 0.770 vs 0.740 ms; 512 beams (256 MiB) 1.472 vs 1.396 ms.
#include <algorithm>
#include <cstring>

#include "spx_internal.h"

using namespace spx;

namespace {

constexpr size_t kChunkBytes = size_t(16) << 20;
constexpr size_t kZeroCopyMaxBytes = 7 * kChunkBytes;
constexpr int kInSlots = 3, kOutSlots = 2;

size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

spx_status ensure_pipeline(spx_ctx* ctx, size_t bytes, size_t n_events) {
  cudaError_t e = cudaSuccess;
  if (!ctx->copy_in) e = cudaStreamCreateWithFlags(&ctx->copy_in, cudaStreamNonBlocking);
  if (e == cudaSuccess && !ctx->copy_out) e = cudaStreamCreateWithFlags(&ctx->copy_out, cudaStreamNonBlocking);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "spx_fft_peaks_host: stream creation");
  if (ctx->stage_bytes < bytes) {
    if (ctx->d_stage) cudaFree(ctx->d_stage);
    ctx->d_stage = nullptr;
    ctx->stage_bytes = 0;
    e = cudaMalloc(&ctx->d_stage, bytes);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "spx_fft_peaks_host: staging buffer");
    ctx->stage_bytes = bytes;
  }
  while (ctx->events.size() < n_events) {
    cudaEvent_t ev;
    e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "spx_fft_peaks_host: event creation");
    ctx->events.push_back(ev);
  }
  return SPX_OK;
}

}  // namespace

extern "C" spx_status spx_fft_peaks_host(spx_ctx* ctx, const void* h_in, uint32_t beams,
                                         uint32_t n_point, uint32_t nfft, uint32_t window,
                                         const spx_peak_params* params, spx_max_value* h_out,
                                         uint32_t* h_counts) {
  if (!ctx) return SPX_ERR_INVALID_ARG;
  if (!params) return fail(ctx, SPX_ERR_INVALID_ARG, "params is null");
  if (params->mode > SPX_PEAK_TOPK)
    return fail(ctx, SPX_ERR_INVALID_ARG, "unknown peak mode " + std::to_string(params->mode));
  if (beams == 0) return SPX_OK;
  if (!h_in) return fail(ctx, SPX_ERR_INVALID_ARG, "spx_fft_peaks_host: null host pointer");
  if (n_point == 0 || nfft < n_point)
    return fail(ctx, SPX_ERR_INVALID_ARG, "spx_fft_peaks_host: need 0 < n_point <= nfft");
  const bool counted = params->mode == SPX_PEAK_ALL || params->mode == SPX_PEAK_TOPK;
  if (counted && !h_counts) return fail(ctx, SPX_ERR_INVALID_ARG, "spx_fft_peaks_host: counts is null");
  // rows per beam in the output
  uint32_t per = 0;
  switch (params->mode) {
    case SPX_PEAK_ONE: per = 4; break;
    case SPX_PEAK_TWO: per = 8; break;
    case SPX_PEAK_ALL: {
      uint32_t s = 0, e = 0;
      spx_all_maxima_capacity(nfft, params->search_start, params->search_end, params->max_per_beam, &s, &e, &per);
      break;
    }
    default: per = params->max_per_beam; break;
  }
  // the output may be null only when it has no rows (ALL with a zero capacity)
  if (!h_out && per > 0) return fail(ctx, SPX_ERR_INVALID_ARG, "spx_fft_peaks_host: null host pointer");
  DeviceGuard guard(ctx->device);
  auto device_view = [](const void* p) -> void* {
    cudaPointerAttributes a{};
    const bool ok = p && cudaPointerGetAttributes(&a, p) == cudaSuccess && a.type == cudaMemoryTypeHost;
    cudaGetLastError();
    return ok ? a.devicePointer : nullptr;
  };
  cudaPointerAttributes pa{};
  pa.devicePointer = device_view(h_in);
  const size_t beam_in = (size_t)n_point * sizeof(float2);
  // mapped input up to kZeroCopyMaxBytes: the kernel reads it over the host link
  const bool zero_copy = pa.devicePointer != nullptr && (size_t)beams * beam_in <= kZeroCopyMaxBytes;
  void* dv_out = device_view(h_out);
  void* dv_cnt = counted ? device_view(h_counts) : nullptr;
  const bool out_in_place = dv_out && (!counted || dv_cnt);
  if (zero_copy && out_in_place) {  // everything in place
    ctx->input_on_host = true;
    spx_status st0 = spx_fft_peaks(ctx, pa.devicePointer, beams, n_point, nfft, window, params,
                                   static_cast<spx_max_value*>(dv_out), static_cast<uint32_t*>(dv_cnt));
    ctx->input_on_host = false;
    if (st0 != SPX_OK) return st0;
    return spx_synchronize(ctx);
  }
  if (zero_copy) {  // results come back in one copy
    const size_t out_bytes = align_up((size_t)beams * std::max<uint32_t>(per, 1) * sizeof(spx_max_value), 256);
    spx_status st0 = ensure_pipeline(ctx, out_bytes + (size_t)beams * sizeof(uint32_t), 0);
    if (st0 != SPX_OK) return st0;
    char* o = static_cast<char*>(ctx->d_stage);
    uint32_t* c = reinterpret_cast<uint32_t*>(o + out_bytes);
    ctx->input_on_host = true;
    st0 = spx_fft_peaks(ctx, pa.devicePointer, beams, n_point, nfft, window, params,
                        reinterpret_cast<spx_max_value*>(o), counted ? c : nullptr);
    ctx->input_on_host = false;
    if (st0 != SPX_OK) return st0;
    cudaError_t e0 = per == 0 ? cudaSuccess
                              : cudaMemcpyAsync(h_out, o, (size_t)beams * per * sizeof(spx_max_value),
                                                cudaMemcpyDeviceToHost, ctx->stream);
    if (e0 == cudaSuccess && counted)
      e0 = cudaMemcpyAsync(h_counts, c, (size_t)beams * sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->stream);
    if (e0 != cudaSuccess) return cuda_fail(ctx, e0, "spx_fft_peaks_host: read-back");
    return spx_synchronize(ctx);
  }
  const uint32_t cb = (uint32_t)std::max<size_t>(1, std::min<size_t>(beams, kChunkBytes / beam_in));
  const uint32_t nchunks = (beams + cb - 1) / cb;
  const size_t in_slot = align_up((size_t)cb * beam_in, 256);
  const size_t out_slot = align_up((size_t)cb * std::max<uint32_t>(per, 1) * sizeof(spx_max_value), 256);
  const size_t cnt_slot = align_up((size_t)cb * sizeof(uint32_t), 256);
  const size_t total = kInSlots * in_slot + (out_in_place ? 0 : kOutSlots * (out_slot + cnt_slot));
  spx_status st = ensure_pipeline(ctx, total, (size_t)3 * nchunks);
  if (st != SPX_OK) return st;
  char* base = static_cast<char*>(ctx->d_stage);
  auto in_ptr = [&](uint32_t i) { return base + (i % kInSlots) * in_slot; };
  auto out_ptr = [&](uint32_t i) { return base + kInSlots * in_slot + (i % kOutSlots) * (out_slot + cnt_slot); };
  cudaEvent_t* ev_in = ctx->events.data();
  cudaEvent_t* ev_comp = ev_in + nchunks;
  cudaEvent_t* ev_out = ev_comp + nchunks;
  // the staging buffer may still be read by work queued before this call
  cudaError_t e = cudaEventRecord(ev_comp[0], ctx->stream);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(ctx->copy_in, ev_comp[0], 0);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "spx_fft_peaks_host: ordering");
  const char* src = static_cast<const char*>(h_in);
  for (uint32_t i = 0; i < nchunks; ++i) {
    const uint32_t b0 = i * cb, nb = std::min(cb, beams - b0);
    if (i >= (uint32_t)kInSlots) e = cudaStreamWaitEvent(ctx->copy_in, ev_comp[i - kInSlots], 0);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(in_ptr(i), src + (size_t)b0 * beam_in, (size_t)nb * beam_in, cudaMemcpyHostToDevice,
                          ctx->copy_in);
    if (e == cudaSuccess) e = cudaEventRecord(ev_in[i], ctx->copy_in);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(ctx->stream, ev_in[i], 0);
    if (e == cudaSuccess && !out_in_place && i >= (uint32_t)kOutSlots)
      e = cudaStreamWaitEvent(ctx->stream, ev_out[i - kOutSlots], 0);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "spx_fft_peaks_host: upload");
    char* o = nullptr;
    uint32_t* c = nullptr;
    if (out_in_place) {  // the kernel writes this chunk's rows into the mapped output
      o = reinterpret_cast<char*>(static_cast<spx_max_value*>(dv_out) + (size_t)b0 * per);
      if (counted) c = static_cast<uint32_t*>(dv_cnt) + b0;
    } else {
      o = out_ptr(i);
      c = reinterpret_cast<uint32_t*>(o + out_slot);
    }
    st = spx_fft_peaks(ctx, in_ptr(i), nb, n_point, nfft, window, params, reinterpret_cast<spx_max_value*>(o),
                       counted ? c : nullptr);
    if (st != SPX_OK) {
      cudaStreamSynchronize(ctx->copy_in);
      return st;
    }
    e = cudaEventRecord(ev_comp[i], ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "spx_fft_peaks_host: ordering");
    if (out_in_place) continue;
    e = cudaStreamWaitEvent(ctx->copy_out, ev_comp[i], 0);
    if (e == cudaSuccess && per > 0)
      e = cudaMemcpyAsync(h_out + (size_t)b0 * per, o, (size_t)nb * per * sizeof(spx_max_value),
                          cudaMemcpyDeviceToHost, ctx->copy_out);
    if (e == cudaSuccess && counted)
      e = cudaMemcpyAsync(h_counts + b0, c, (size_t)nb * sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->copy_out);
    if (e == cudaSuccess) e = cudaEventRecord(ev_out[i], ctx->copy_out);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "spx_fft_peaks_host: read-back");
  }
  e = cudaStreamSynchronize(ctx->copy_out);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "spx_fft_peaks_host: synchronize");
  return spx_synchronize(ctx);
}
