// facade.cpp — the C++ classes of include/spectrum_gb300/spectrum.hpp on top
// of the C ABI.  Each method follows the reference method it replaces (cited
// per method) for validation, defaults, batching and result layout; the
// device work is one or two spx_* calls on the backend's stream.
#include "spectrum_gb300/spectrum.hpp"

#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstring>
#include <functional>
#include <stdexcept>
#include <type_traits>

namespace spectrum_gb300 {

Context::Context(drv_gpu_lib::IBackend* backend) {
  if (!backend) throw std::invalid_argument("backend cannot be null");
  device_ = backend->GetDeviceIndex();
  spx_status st = spx_create(device_, &ctx_);
  if (st != SPX_OK) throw std::runtime_error(std::string("spx_create: ") + spx_status_string(st));
  spx_set_stream(ctx_, backend->GetNativeStream());
}

Context::~Context() {
  if (ctx_) spx_destroy(ctx_);
}

void Context::check(spx_status st, const char* where) const {
  if (st == SPX_OK) return;
  std::string msg = std::string(where) + ": " + spx_status_string(st) + ": " + spx_last_error(ctx_);
  if (st == SPX_ERR_INVALID_ARG) throw std::invalid_argument(msg);
  throw std::runtime_error(msg);
}

DeviceBuffer::~DeviceBuffer() {
  if (ptr_) cudaFree(ptr_);
}

void* DeviceBuffer::ensure(size_t bytes, const char* where) {
  if (bytes <= bytes_ && ptr_) return ptr_;
  if (ptr_) cudaFree(ptr_);
  ptr_ = nullptr;
  bytes_ = 0;
  cudaError_t e = cudaMalloc(&ptr_, std::max<size_t>(bytes, 256));
  if (e != cudaSuccess) {
    cudaGetLastError();
    throw std::runtime_error(std::string(where) + ": cudaMalloc failed: " + cudaGetErrorString(e));
  }
  bytes_ = std::max<size_t>(bytes, 256);
  return ptr_;
}

namespace {

void cuda_check(cudaError_t e, const char* where) {
  if (e != cudaSuccess) throw std::runtime_error(std::string(where) + ": " + cudaGetErrorString(e));
}

// Beams per batch for a per-beam footprint within memory_limit of the free
// device memory (the reference's BatchManager::CalculateOptimalBatchSize).
size_t batch_beams(size_t beams, size_t bytes_per_beam, float memory_limit, size_t external = 0) {
  size_t free_b = 0, total_b = 0;
  if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) return beams;
  const double budget = std::max(0.0, (double)free_b * std::clamp(memory_limit, 0.0f, 1.0f) - (double)external);
  const size_t fit = bytes_per_beam ? (size_t)(budget / (double)bytes_per_beam) : beams;
  return std::max<size_t>(1, std::min(beams, fit));
}

// Events around stages of a call on one stream.
struct StageTimer {
  cudaStream_t s;
  std::vector<cudaEvent_t> ev;
  explicit StageTimer(void* stream) : s(static_cast<cudaStream_t>(stream)) {}
  ~StageTimer() {
    for (auto e : ev) cudaEventDestroy(e);
  }
  size_t mark() {
    cudaEvent_t e;
    cudaEventCreate(&e);
    cudaEventRecord(e, s);
    ev.push_back(e);
    return ev.size() - 1;
  }
  double ms(size_t a, size_t b) const {
    float t = 0.f;
    cudaEventElapsedTime(&t, ev[a], ev[b]);
    return t;
  }
};

uint32_t checked_nfft(uint32_t n_point, uint32_t repeat_count, const char* where) {
  if (n_point == 0) throw std::invalid_argument(std::string(where) + ": n_point must be > 0");
  if (repeat_count == 0) throw std::invalid_argument(std::string(where) + ": repeat_count must be > 0");
  const uint64_t n = (uint64_t)spx_next_pow2(n_point) * repeat_count;
  if (n > 0xffffffffull || !spx_fft_size_supported((uint32_t)n))
    throw std::invalid_argument(std::string(where) + ": nFFT " + std::to_string(n) +
                                " is not a transform size of this build (any length 2 .. 2^27; 2^a 3^b up to 2^28"
                                " with a split into two factors <= 16384)");
  return (uint32_t)n;
}

}  // namespace
}  // namespace spectrum_gb300

// ===========================================================================
// fft_processor
// ===========================================================================
namespace fft_processor {

using spectrum_gb300::Context;
using spectrum_gb300::DeviceBuffer;

struct FFTProcessorGB300::Impl {
  explicit Impl(drv_gpu_lib::IBackend* b) : ctx(b), stream(b->GetNativeStream()) {}
  Context ctx;
  void* stream;
  DeviceBuffer in, out;
};

FFTProcessorGB300::FFTProcessorGB300(drv_gpu_lib::IBackend* backend) : impl_(new Impl(backend)) {}
FFTProcessorGB300::~FFTProcessorGB300() = default;
FFTProcessorGB300::FFTProcessorGB300(FFTProcessorGB300&&) noexcept = default;
FFTProcessorGB300& FFTProcessorGB300::operator=(FFTProcessorGB300&&) noexcept = default;

namespace {
template <class R>
constexpr bool is_complex_result() {
  return std::is_same<R, FFTComplexResult>::value;
}
}  // namespace

// FFTProcessorROCm::ProcessComplex / ProcessMagPhase (fft_processor_rocm.cpp:306-560):
// nFFT = nextPow2(n_point) * repeat_count, no window, batches within
// memory_limit, results per beam with the absolute beam id.
template <class R>
std::vector<R> FFTProcessorGB300::run(const std::complex<float>* host, void* gpu, const FFTProcessorParams& params,
                                      ROCmProfEvents* prof_events) {
  const char* where = is_complex_result<R>() ? "ProcessComplex" : "ProcessMagPhase";
  nFFT_ = spectrum_gb300::checked_nfft(params.n_point, params.repeat_count, where);
  const uint32_t nfft = nFFT_;
  const bool cplx = is_complex_result<R>();
  const bool freq = !cplx && params.output_mode == FFTOutputMode::MAGNITUDE_PHASE_FREQ;
  const size_t in_beam = (size_t)params.n_point * sizeof(std::complex<float>);
  const size_t out_beam = (size_t)nfft * 8;  // complex64 or {mag, phase}
  const size_t nb = spectrum_gb300::batch_beams(params.beam_count, in_beam + out_beam, params.memory_limit);
  Context& c = impl_->ctx;
  std::vector<R> results;
  results.reserve(params.beam_count);
  std::vector<float> raw;
  prof_ = FFTProfilingData{};
  const auto t_start = std::chrono::steady_clock::now();
  for (size_t b0 = 0; b0 < params.beam_count; b0 += nb) {
    const size_t cnt = std::min(nb, (size_t)params.beam_count - b0);
    spectrum_gb300::StageTimer tm(impl_->stream);
    const void* d_in;
    size_t m0 = tm.mark();
    if (host) {
      void* d = impl_->in.ensure(cnt * in_beam, where);
      spectrum_gb300::cuda_check(cudaMemcpyAsync(d, host + b0 * params.n_point, cnt * in_beam,
                                                 cudaMemcpyHostToDevice, static_cast<cudaStream_t>(impl_->stream)),
                                 where);
      d_in = d;
    } else {
      d_in = static_cast<const char*>(gpu) + b0 * in_beam;
    }
    size_t m1 = tm.mark();
    void* d_out = impl_->out.ensure(cnt * out_beam, where);
    c.check(spx_fft(c.get(), d_in, (uint32_t)cnt, params.n_point, nfft, SPX_WINDOW_NONE,
                    cplx ? SPX_OUT_COMPLEX : SPX_OUT_MAGPHASE, 1.0f, d_out),
            where);
    size_t m2 = tm.mark();
    raw.resize(cnt * nfft * 2);
    spectrum_gb300::cuda_check(cudaMemcpyAsync(raw.data(), d_out, cnt * out_beam, cudaMemcpyDeviceToHost,
                                               static_cast<cudaStream_t>(impl_->stream)),
                               where);
    size_t m3 = tm.mark();
    spectrum_gb300::cuda_check(cudaStreamSynchronize(static_cast<cudaStream_t>(impl_->stream)), where);
    c.check(spx_synchronize(c.get()), where);
    prof_.upload_time_ms += tm.ms(m0, m1);
    prof_.fft_time_ms += tm.ms(m1, m2);
    prof_.download_time_ms += tm.ms(m2, m3);
    if (prof_events) {
      prof_events->push_back({"Upload", {tm.ms(m0, m1), host ? "H2D" : "device input"}});
      prof_events->push_back({"FFT", {tm.ms(m1, m2), cplx ? "spx_fft (complex)" : "spx_fft (mag+phase)"}});
      prof_events->push_back({"Download", {tm.ms(m2, m3), "D2H"}});
    }
    for (size_t i = 0; i < cnt; ++i) {
      R r;
      r.beam_id = (uint32_t)(b0 + i);
      r.nFFT = nfft;
      r.sample_rate = params.sample_rate;
      const float* src = raw.data() + i * (size_t)nfft * 2;
      if constexpr (is_complex_result<R>()) {
        r.spectrum.resize(nfft);
        // std::complex<float> has the layout of float[2] (array-oriented access)
        std::memcpy(static_cast<void*>(r.spectrum.data()), src, (size_t)nfft * 8);
      } else {
        r.magnitude.resize(nfft);
        r.phase.resize(nfft);
        for (uint32_t k = 0; k < nfft; ++k) {
          r.magnitude[k] = src[2 * k];
          r.phase[k] = src[2 * k + 1];
        }
        if (freq) {  // fft_processor_rocm.cpp:289-295
          r.frequency.resize(nfft);
          const float step = params.sample_rate / static_cast<float>(nfft);
          for (uint32_t k = 0; k < nfft; ++k) r.frequency[k] = static_cast<float>(k) * step;
        }
      }
      results.push_back(std::move(r));
    }
  }
  prof_.total_time_ms =
      std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_start).count();
  return results;
}

std::vector<FFTComplexResult> FFTProcessorGB300::ProcessComplex(const std::vector<std::complex<float>>& data,
                                                                const FFTProcessorParams& params,
                                                                ROCmProfEvents* prof_events) {
  const size_t expected = (size_t)params.beam_count * params.n_point;
  if (data.size() != expected)
    throw std::invalid_argument("ProcessComplex: input size " + std::to_string(data.size()) + " != expected " +
                                std::to_string(expected));
  return run<FFTComplexResult>(data.data(), nullptr, params, prof_events);
}

std::vector<FFTComplexResult> FFTProcessorGB300::ProcessComplex(void* gpu_data, const FFTProcessorParams& params,
                                                                size_t gpu_memory_bytes) {
  if (!gpu_data) throw std::invalid_argument("ProcessComplex: gpu_data is null");
  const size_t need = (size_t)params.beam_count * params.n_point * 8;
  if (gpu_memory_bytes && gpu_memory_bytes < need)
    throw std::invalid_argument("ProcessComplex: gpu_memory_bytes " + std::to_string(gpu_memory_bytes) +
                                " < " + std::to_string(need));
  return run<FFTComplexResult>(nullptr, gpu_data, params, nullptr);
}

std::vector<FFTMagPhaseResult> FFTProcessorGB300::ProcessMagPhase(const std::vector<std::complex<float>>& data,
                                                                  const FFTProcessorParams& params,
                                                                  ROCmProfEvents* prof_events) {
  const size_t expected = (size_t)params.beam_count * params.n_point;
  if (data.size() != expected)
    throw std::invalid_argument("ProcessMagPhase: input size " + std::to_string(data.size()) + " != expected " +
                                std::to_string(expected));
  return run<FFTMagPhaseResult>(data.data(), nullptr, params, prof_events);
}

std::vector<FFTMagPhaseResult> FFTProcessorGB300::ProcessMagPhase(void* gpu_data, const FFTProcessorParams& params,
                                                                  size_t gpu_memory_bytes) {
  if (!gpu_data) throw std::invalid_argument("ProcessMagPhase: gpu_data is null");
  const size_t need = (size_t)params.beam_count * params.n_point * 8;
  if (gpu_memory_bytes && gpu_memory_bytes < need)
    throw std::invalid_argument("ProcessMagPhase: gpu_memory_bytes " + std::to_string(gpu_memory_bytes) +
                                " < " + std::to_string(need));
  return run<FFTMagPhaseResult>(nullptr, gpu_data, params, nullptr);
}

// FFTProcessorROCm::ProcessMagnitudesToGPU (fft_processor_rocm.cpp:585-659):
// window + pad + FFT + |X| (or |X|^2) with inv_n = 1 into the caller buffer;
// here spx_fft with its |X| epilogue (no separate pad or magnitude pass).
void FFTProcessorGB300::ProcessMagnitudesToGPU(void* gpu_data, void* gpu_out_magnitudes,
                                               const FFTProcessorParams& params, bool squared, WindowType window,
                                               ROCmProfEvents* prof_events) {
  if (!gpu_data) throw std::invalid_argument("ProcessMagnitudesToGPU: gpu_data is null");
  if (!gpu_out_magnitudes) throw std::invalid_argument("ProcessMagnitudesToGPU: gpu_out_magnitudes is null");
  nFFT_ = spectrum_gb300::checked_nfft(params.n_point, params.repeat_count, "ProcessMagnitudesToGPU");
  Context& c = impl_->ctx;
  spectrum_gb300::StageTimer tm(impl_->stream);
  size_t m0 = tm.mark();
  c.check(spx_fft(c.get(), gpu_data, params.beam_count, params.n_point, nFFT_, static_cast<uint32_t>(window),
                  squared ? SPX_OUT_MAG2 : SPX_OUT_MAG, 1.0f, gpu_out_magnitudes),
          "ProcessMagnitudesToGPU");
  size_t m1 = tm.mark();
  c.check(spx_synchronize(c.get()), "ProcessMagnitudesToGPU");
  prof_ = FFTProfilingData{};
  prof_.fft_time_ms = tm.ms(m0, m1);
  prof_.total_time_ms = prof_.fft_time_ms;
  if (prof_events)
    prof_events->push_back({"FFT+Magnitude", {tm.ms(m0, m1), squared ? "spx_fft (|X|^2)" : "spx_fft (|X|)"}});
}

// ---- ComplexToMagPhase (complex_to_mag_phase_rocm.cpp:170-410) -----------
struct ComplexToMagPhaseGB300::Impl {
  explicit Impl(drv_gpu_lib::IBackend* b) : ctx(b), stream(b->GetNativeStream()) {}
  Context ctx;
  void* stream;
  DeviceBuffer in, out;
  cudaStream_t s() const { return static_cast<cudaStream_t>(stream); }
};

ComplexToMagPhaseGB300::ComplexToMagPhaseGB300(drv_gpu_lib::IBackend* backend) : impl_(new Impl(backend)) {}
ComplexToMagPhaseGB300::~ComplexToMagPhaseGB300() = default;
ComplexToMagPhaseGB300::ComplexToMagPhaseGB300(ComplexToMagPhaseGB300&&) noexcept = default;
ComplexToMagPhaseGB300& ComplexToMagPhaseGB300::operator=(ComplexToMagPhaseGB300&&) noexcept = default;

float ComplexToMagPhaseGB300::ComputeInvN(const MagPhaseParams& params) {
  if (params.norm_coeff < 0.0f) return params.n_point > 0 ? 1.0f / static_cast<float>(params.n_point) : 1.0f;
  if (params.norm_coeff > 0.0f) return params.norm_coeff;
  return 1.0f;
}

namespace {
std::vector<MagPhaseResult> split_mag_phase(const std::vector<float>& raw, size_t beams, size_t b0, uint32_t n) {
  std::vector<MagPhaseResult> out;
  out.reserve(beams);
  for (size_t i = 0; i < beams; ++i) {
    MagPhaseResult r;
    r.beam_id = (uint32_t)(b0 + i);
    r.n_point = n;
    r.magnitude.resize(n);
    r.phase.resize(n);
    for (uint32_t k = 0; k < n; ++k) {
      r.magnitude[k] = raw[(i * n + k) * 2];
      r.phase[k] = raw[(i * n + k) * 2 + 1];
    }
    out.push_back(std::move(r));
  }
  return out;
}
}  // namespace

std::vector<MagPhaseResult> ComplexToMagPhaseGB300::Process(const std::vector<std::complex<float>>& data,
                                                            const MagPhaseParams& params) {
  const size_t expected = (size_t)params.beam_count * params.n_point;
  if (data.size() != expected)
    throw std::invalid_argument("C2MP::Process: input size " + std::to_string(data.size()) + " != expected " +
                                std::to_string(expected));
  const size_t per = (size_t)params.n_point * 16;
  const size_t nb = spectrum_gb300::batch_beams(params.beam_count, per, params.memory_limit);
  std::vector<MagPhaseResult> all;
  all.reserve(params.beam_count);
  std::vector<float> raw;
  for (size_t b0 = 0; b0 < params.beam_count; b0 += nb) {
    const size_t cnt = std::min(nb, (size_t)params.beam_count - b0), total = cnt * params.n_point;
    void* d_in = impl_->in.ensure(total * 8, "C2MP::Process");
    void* d_out = impl_->out.ensure(total * 8, "C2MP::Process");
    spectrum_gb300::cuda_check(
        cudaMemcpyAsync(d_in, data.data() + b0 * params.n_point, total * 8, cudaMemcpyHostToDevice, impl_->s()),
        "C2MP::Process");
    impl_->ctx.check(spx_mag_phase(impl_->ctx.get(), d_in, d_out, total), "C2MP::Process");
    raw.resize(total * 2);
    spectrum_gb300::cuda_check(cudaMemcpyAsync(raw.data(), d_out, total * 8, cudaMemcpyDeviceToHost, impl_->s()),
                               "C2MP::Process");
    spectrum_gb300::cuda_check(cudaStreamSynchronize(impl_->s()), "C2MP::Process");
    auto br = split_mag_phase(raw, cnt, b0, params.n_point);
    for (auto& r : br) all.push_back(std::move(r));
  }
  return all;
}

std::vector<MagPhaseResult> ComplexToMagPhaseGB300::Process(void* gpu_data, const MagPhaseParams& params,
                                                            size_t gpu_memory_bytes) {
  if (!gpu_data) throw std::invalid_argument("C2MP::Process: gpu_data is null");
  const size_t per = (size_t)params.n_point * 8;
  const size_t external = gpu_memory_bytes ? gpu_memory_bytes : (size_t)params.beam_count * params.n_point * 8;
  const size_t nb = spectrum_gb300::batch_beams(params.beam_count, per, params.memory_limit, external);
  std::vector<MagPhaseResult> all;
  all.reserve(params.beam_count);
  std::vector<float> raw;
  for (size_t b0 = 0; b0 < params.beam_count; b0 += nb) {
    const size_t cnt = std::min(nb, (size_t)params.beam_count - b0), total = cnt * params.n_point;
    void* d_out = impl_->out.ensure(total * 8, "C2MP::Process");
    impl_->ctx.check(spx_mag_phase(impl_->ctx.get(), static_cast<const char*>(gpu_data) + b0 * params.n_point * 8,
                                   d_out, total),
                     "C2MP::Process");
    raw.resize(total * 2);
    spectrum_gb300::cuda_check(cudaMemcpyAsync(raw.data(), d_out, total * 8, cudaMemcpyDeviceToHost, impl_->s()),
                               "C2MP::Process");
    spectrum_gb300::cuda_check(cudaStreamSynchronize(impl_->s()), "C2MP::Process");
    auto br = split_mag_phase(raw, cnt, b0, params.n_point);
    for (auto& r : br) all.push_back(std::move(r));
  }
  return all;
}

void* ComplexToMagPhaseGB300::ProcessToGPU(const std::vector<std::complex<float>>& data,
                                           const MagPhaseParams& params) {
  const size_t total = (size_t)params.beam_count * params.n_point;
  if (data.size() != total) throw std::invalid_argument("C2MP::ProcessToGPU: input size mismatch");
  void* d_in = impl_->in.ensure(total * 8, "C2MP ProcessToGPU");
  spectrum_gb300::cuda_check(cudaMemcpyAsync(d_in, data.data(), total * 8, cudaMemcpyHostToDevice, impl_->s()),
                             "C2MP ProcessToGPU: H2D");
  return ProcessToGPU(d_in, params, total * 8);
}

void* ComplexToMagPhaseGB300::ProcessToGPU(void* gpu_data, const MagPhaseParams& params, size_t) {
  if (!gpu_data) throw std::invalid_argument("C2MP::ProcessToGPU: gpu_data is null");
  const size_t total = (size_t)params.beam_count * params.n_point;
  void* out = nullptr;
  cudaError_t e = cudaMalloc(&out, std::max<size_t>(total * 8, 8));
  if (e != cudaSuccess) throw std::runtime_error("C2MP ProcessToGPU: cudaMalloc output failed");
  const spx_status st = spx_mag_phase(impl_->ctx.get(), gpu_data, out, total);
  if (st == SPX_OK) e = cudaStreamSynchronize(impl_->s());
  if (st != SPX_OK || e != cudaSuccess) {
    cudaFree(out);
    impl_->ctx.check(st != SPX_OK ? st : SPX_ERR_CUDA, "C2MP ProcessToGPU");
  }
  return out;  // caller owns
}

std::vector<MagnitudeResult> ComplexToMagPhaseGB300::ProcessMagnitude(void* gpu_data, const MagPhaseParams& params,
                                                                      size_t) {
  if (!gpu_data) throw std::invalid_argument("C2MP::ProcessMagnitude: gpu_data is null");
  const size_t total = (size_t)params.beam_count * params.n_point;
  void* d_out = impl_->out.ensure(total * 4, "C2MP::ProcessMagnitude");
  impl_->ctx.check(spx_magnitude(impl_->ctx.get(), gpu_data, static_cast<float*>(d_out), total, ComputeInvN(params), 0),
                   "C2MP::ProcessMagnitude");
  std::vector<float> raw(total);
  spectrum_gb300::cuda_check(cudaMemcpyAsync(raw.data(), d_out, total * 4, cudaMemcpyDeviceToHost, impl_->s()),
                             "C2MP::ProcessMagnitude");
  spectrum_gb300::cuda_check(cudaStreamSynchronize(impl_->s()), "C2MP::ProcessMagnitude");
  std::vector<MagnitudeResult> out(params.beam_count);
  for (uint32_t b = 0; b < params.beam_count; ++b) {
    out[b].beam_id = b;
    out[b].n_point = params.n_point;
    out[b].magnitude.assign(raw.begin() + (size_t)b * params.n_point, raw.begin() + (size_t)(b + 1) * params.n_point);
  }
  return out;
}

void* ComplexToMagPhaseGB300::ProcessMagnitudeToGPU(void* gpu_data, const MagPhaseParams& params, size_t) {
  if (!gpu_data) throw std::invalid_argument("C2MP::ProcessMagnitudeToGPU: gpu_data is null");
  const size_t total = (size_t)params.beam_count * params.n_point;
  void* out = nullptr;
  if (cudaMalloc(&out, std::max<size_t>(total * 4, 4)) != cudaSuccess)
    throw std::runtime_error("C2MP ProcessMagnitudeToGPU: cudaMalloc failed");
  const spx_status st = spx_magnitude(impl_->ctx.get(), gpu_data, static_cast<float*>(out), total, ComputeInvN(params), 0);
  cudaError_t e = st == SPX_OK ? cudaStreamSynchronize(impl_->s()) : cudaSuccess;
  if (st != SPX_OK || e != cudaSuccess) {
    cudaFree(out);
    impl_->ctx.check(st != SPX_OK ? st : SPX_ERR_CUDA, "C2MP ProcessMagnitudeToGPU");
  }
  return out;  // caller owns
}

void ComplexToMagPhaseGB300::ProcessMagnitudeToBuffer(void* gpu_complex_in, void* gpu_magnitude_out,
                                                      const MagPhaseParams& params) {
  if (!gpu_complex_in || !gpu_magnitude_out)
    throw std::invalid_argument("C2MP::ProcessMagnitudeToBuffer: null pointer");
  const size_t total = (size_t)params.beam_count * params.n_point;
  impl_->ctx.check(spx_magnitude(impl_->ctx.get(), gpu_complex_in, static_cast<float*>(gpu_magnitude_out), total,
                                 ComputeInvN(params), 0),
                   "C2MP::ProcessMagnitudeToBuffer");
  spectrum_gb300::cuda_check(cudaStreamSynchronize(impl_->s()), "C2MP::ProcessMagnitudeToBuffer");
}

}  // namespace fft_processor

// ===========================================================================
// antenna_fft
// ===========================================================================
namespace antenna_fft {

using spectrum_gb300::Context;

namespace {

// Reads counts (and maxima for CPU / ALL) into the reference's result shape
// (all_maxima_pipeline_rocm.cpp:397-460): per-beam counts truncated to the
// capacity on the host side, total_maxima of what was returned (untruncated
// counts for GPU-only), device buffers handed to the caller for GPU / ALL.
AllMaximaResult make_result(Context& c, void* d_out, void* d_counts, uint32_t beams, uint32_t cap,
                            OutputDestination dest) {
  cudaStream_t s = static_cast<cudaStream_t>(spx_get_stream(c.get()));
  std::vector<uint32_t> counts(beams);
  cudaError_t e = cudaMemcpyAsync(counts.data(), d_counts, (size_t)beams * 4, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    cudaFree(d_out);
    cudaFree(d_counts);
    throw std::runtime_error(std::string("AllMaximaPipeline: read beam_counts failed: ") + cudaGetErrorString(e));
  }
  AllMaximaResult r;
  r.destination = dest;
  if (dest == OutputDestination::CPU || dest == OutputDestination::ALL) {
    r.beams.resize(beams);
    std::vector<spx_max_value> all((size_t)beams * cap);
    if (cap) e = cudaMemcpy(all.data(), d_out, all.size() * sizeof(spx_max_value), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
      cudaFree(d_out);
      cudaFree(d_counts);
      throw std::runtime_error("AllMaximaPipeline: read maxima failed");
    }
    for (uint32_t b = 0; b < beams; ++b) {
      const uint32_t n = std::min(counts[b], cap);
      r.beams[b].antenna_id = b;
      r.beams[b].num_maxima = n;
      r.total_maxima += n;
      r.beams[b].maxima.resize(n);
      if (n) std::memcpy(r.beams[b].maxima.data(), all.data() + (size_t)b * cap, n * sizeof(MaxValue));
    }
  } else {
    for (uint32_t b = 0; b < beams; ++b) r.total_maxima += counts[b];
  }
  if (dest == OutputDestination::GPU || dest == OutputDestination::ALL) {
    r.gpu_maxima = d_out;
    r.gpu_counts = d_counts;
    r.gpu_bytes = (size_t)beams * cap * sizeof(MaxValue);
  } else {
    cudaFree(d_out);
    cudaFree(d_counts);
  }
  return r;
}

void alloc_outputs(uint32_t beams, uint32_t cap, void** d_out, void** d_counts) {
  *d_out = *d_counts = nullptr;
  if (cudaMalloc(d_out, std::max<size_t>((size_t)beams * cap * sizeof(MaxValue), 32)) != cudaSuccess ||
      cudaMalloc(d_counts, std::max<size_t>((size_t)beams * 4, 4)) != cudaSuccess) {
    cudaFree(*d_out);
    cudaGetLastError();
    throw std::runtime_error("AllMaximaPipeline: cudaMalloc of the outputs failed");
  }
}

}  // namespace

AllMaximaPipelineGB300::AllMaximaPipelineGB300(drv_gpu_lib::IBackend* backend)
    : ctx_(new Context(backend)) {}
AllMaximaPipelineGB300::~AllMaximaPipelineGB300() = default;

// AllMaximaPipelineROCm::Execute (all_maxima_pipeline_rocm.cpp:258-472).
AllMaximaResult AllMaximaPipelineGB300::Execute(void* magnitudes_gpu, void* fft_data_gpu, uint32_t beam_count,
                                                uint32_t nFFT, float sample_rate, OutputDestination dest,
                                                uint32_t search_start, uint32_t search_end,
                                                size_t max_maxima_per_beam) {
  if (!fft_data_gpu) throw std::invalid_argument("AllMaximaPipeline: fft_data_gpu is null");
  uint32_t s = 0, e = 0, cap = 0;
  const uint32_t maxpb = (uint32_t)std::min<size_t>(max_maxima_per_beam, 0xffffffffu);
  ctx_->check((spx_status)spx_all_maxima_capacity(nFFT, search_start, search_end, maxpb, &s, &e, &cap),
              "AllMaximaPipeline");
  void *d_out, *d_counts;
  alloc_outputs(beam_count, cap, &d_out, &d_counts);
  spx_peak_params p{};
  p.mode = SPX_PEAK_ALL;
  p.search_start = search_start;
  p.search_end = search_end;
  p.max_per_beam = maxpb;
  p.refine = SPX_REFINE_NONE;
  p.sample_rate = sample_rate;
  const spx_status st = spx_all_maxima(ctx_->get(), static_cast<const float*>(magnitudes_gpu), fft_data_gpu,
                                       beam_count, nFFT, &p, static_cast<spx_max_value*>(d_out),
                                       static_cast<uint32_t*>(d_counts));
  const spx_status st2 = st == SPX_OK ? spx_synchronize(ctx_->get()) : st;
  if (st2 != SPX_OK) {
    cudaFree(d_out);
    cudaFree(d_counts);
    ctx_->check(st2, "AllMaximaPipeline");
  }
  return make_result(*ctx_, d_out, d_counts, beam_count, cap, dest);
}

// ---- SpectrumProcessor (spectrum_processor_rocm.cpp) ----------------------
SpectrumProcessorGB300::SpectrumProcessorGB300(drv_gpu_lib::IBackend* backend)
    : ctx_(new Context(backend)), pipeline_(backend) {}
SpectrumProcessorGB300::~SpectrumProcessorGB300() = default;

// Initialize + CalculateFFTSize (spectrum_processor_rocm.cpp:111-160, 1137-1143).
void SpectrumProcessorGB300::Initialize(const SpectrumParams& params) {
  params_ = params;
  params_.base_fft = spx_next_pow2(params_.n_point);
  params_.nFFT = spectrum_gb300::checked_nfft(params_.n_point, params_.repeat_count, "SpectrumProcessor::Initialize");
  if (params_.search_range == 0) params_.search_range = params_.nFFT / 4;
  initialized_ = true;
}

size_t SpectrumProcessorGB300::CalculateBytesPerAntenna() const {
  // input + spectrum + 8 MaxValue (the fused path keeps the spectrum on chip
  // where it can; the composed path needs it)
  return (size_t)params_.n_point * 8 + (size_t)params_.nFFT * 8 + 8 * sizeof(MaxValue);
}

void SpectrumProcessorGB300::ReallocateBuffersForBatch(size_t batch_antenna_count) {
  in_.ensure(batch_antenna_count * (size_t)params_.n_point * 8, "ReallocateBuffersForBatch");
  out_.ensure(batch_antenna_count * 8 * sizeof(MaxValue), "ReallocateBuffersForBatch");
}

// ONE_PEAK / TWO_PEAKS on beams already in device memory: spx_fft_peaks
// (windowed, zero-padded FFT, then the post kernel), then ReadResults
// (spectrum_processor_rocm.cpp:1072-1122).
std::vector<SpectrumResult> SpectrumProcessorGB300::peaks_from_device(const void* d_in, size_t beams,
                                                                      size_t start_antenna) {
  if (params_.peak_mode == PeakSearchMode::ALL_MAXIMA)
    throw std::invalid_argument("SpectrumProcessor: ProcessFromCPU/FromGPU need ONE_PEAK or TWO_PEAKS");
  const bool two = params_.peak_mode == PeakSearchMode::TWO_PEAKS;
  const size_t per = two ? 8 : 4;
  void* d_out = out_.ensure(beams * per * sizeof(MaxValue), "ProcessBatch");
  spx_peak_params p{};
  p.mode = two ? SPX_PEAK_TWO : SPX_PEAK_ONE;
  p.search_range = params_.search_range;
  p.sample_rate = params_.sample_rate;
  p.refine = SPX_REFINE_PARABOLIC;
  spectrum_gb300::StageTimer tm(spx_get_stream(ctx_->get()));
  size_t m0 = tm.mark();
  ctx_->check(spx_fft_peaks(ctx_->get(), d_in, (uint32_t)beams, params_.n_point, params_.nFFT, SPX_WINDOW_NONE, &p,
                            static_cast<spx_max_value*>(d_out), nullptr),
              "ProcessBatch");
  size_t m1 = tm.mark();
  std::vector<MaxValue> raw(beams * per);
  spectrum_gb300::cuda_check(cudaMemcpyAsync(raw.data(), d_out, raw.size() * sizeof(MaxValue),
                                             cudaMemcpyDeviceToHost, tm.s),
                             "ReadResults");
  size_t m2 = tm.mark();
  ctx_->check(spx_synchronize(ctx_->get()), "ProcessBatch");
  prof_.fft_time_ms += tm.ms(m0, m1);
  prof_.download_time_ms += tm.ms(m1, m2);
  std::vector<SpectrumResult> results;
  results.reserve(beams * (two ? 2 : 1));
  for (size_t i = 0; i < beams; ++i) {
    for (size_t h = 0; h < (two ? 2u : 1u); ++h) {
      const MaxValue* m = raw.data() + i * per + h * 4;
      SpectrumResult r{};
      r.antenna_id = (uint32_t)(start_antenna + i);
      r.interpolated = m[0];
      r.left_point = m[1];
      r.center_point = m[2];
      r.right_point = m[3];
      results.push_back(r);
    }
  }
  return results;
}

std::vector<SpectrumResult> SpectrumProcessorGB300::ProcessBatch(const std::vector<std::complex<float>>& data,
                                                                 size_t start_antenna, size_t batch_antenna_count) {
  if (!initialized_) throw std::runtime_error("SpectrumProcessor::ProcessBatch: not initialized");
  const size_t off = start_antenna * params_.n_point;
  if (off + batch_antenna_count * params_.n_point > data.size())
    throw std::invalid_argument("SpectrumProcessor::ProcessBatch: batch exceeds the input");
  const size_t bytes = batch_antenna_count * (size_t)params_.n_point * 8;
  void* d_in = in_.ensure(bytes, "ProcessBatch");
  spectrum_gb300::StageTimer tm(spx_get_stream(ctx_->get()));
  size_t m0 = tm.mark();
  spectrum_gb300::cuda_check(cudaMemcpyAsync(d_in, data.data() + off, bytes, cudaMemcpyHostToDevice, tm.s),
                             "UploadData");
  size_t m1 = tm.mark();
  auto r = peaks_from_device(d_in, batch_antenna_count, start_antenna);
  prof_.upload_time_ms += tm.ms(m0, m1);
  return r;
}

std::vector<SpectrumResult> SpectrumProcessorGB300::ProcessBatchFromGPU(void* gpu_data, size_t src_offset_bytes,
                                                                        size_t start_antenna,
                                                                        size_t batch_antenna_count) {
  if (!initialized_) throw std::runtime_error("SpectrumProcessor::ProcessBatchFromGPU: not initialized");
  if (!gpu_data) throw std::invalid_argument("SpectrumProcessor::ProcessBatchFromGPU: gpu_data cannot be null");
  return peaks_from_device(static_cast<const char*>(gpu_data) + src_offset_bytes, batch_antenna_count, start_antenna);
}

// ProcessFromCPU (spectrum_processor_rocm.cpp:263-307): size check, batches
// within memory_limit.
std::vector<SpectrumResult> SpectrumProcessorGB300::ProcessFromCPU(const std::vector<std::complex<float>>& data) {
  if (!initialized_) throw std::runtime_error("SpectrumProcessor::ProcessFromCPU: not initialized");
  const size_t expected = (size_t)params_.antenna_count * params_.n_point;
  if (data.size() != expected)
    throw std::invalid_argument("SpectrumProcessor::ProcessFromCPU: input size mismatch. Expected " +
                                std::to_string(expected) + ", got " + std::to_string(data.size()));
  prof_ = ProfilingData{};
  const auto t0 = std::chrono::steady_clock::now();
  const size_t nb = spectrum_gb300::batch_beams(params_.antenna_count, CalculateBytesPerAntenna(), params_.memory_limit);
  std::vector<SpectrumResult> all;
  for (size_t b0 = 0; b0 < params_.antenna_count; b0 += nb) {
    auto r = ProcessBatch(data, b0, std::min(nb, (size_t)params_.antenna_count - b0));
    all.insert(all.end(), r.begin(), r.end());
  }
  prof_.total_time_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  return all;
}

std::vector<SpectrumResult> SpectrumProcessorGB300::ProcessFromGPU(void* gpu_data, size_t antenna_count,
                                                                   size_t n_point, size_t gpu_memory_bytes) {
  if (!gpu_data) throw std::invalid_argument("SpectrumProcessor::ProcessFromGPU: gpu_data cannot be null");
  if (!initialized_) throw std::runtime_error("SpectrumProcessor::ProcessFromGPU: not initialized");
  if (n_point != params_.n_point)
    throw std::invalid_argument("SpectrumProcessor::ProcessFromGPU: n_point differs from the initialised n_point");
  if (gpu_memory_bytes && gpu_memory_bytes < antenna_count * n_point * 8)
    throw std::invalid_argument("SpectrumProcessor::ProcessFromGPU: gpu_memory_bytes too small");
  prof_ = ProfilingData{};
  return peaks_from_device(gpu_data, antenna_count, 0);
}

// FindAllMaximaFromCPU / FromGPUPipeline (spectrum_processor_rocm.cpp:444-690):
// pad + FFT + |X| + detect/scan/compact with max 1000 per beam, the search
// window from the call; here the FFT and the search run as spx_fft_peaks
// (fused where the transform fits one cluster).
AllMaximaResult SpectrumProcessorGB300::all_maxima_from_device(const void* d_in, size_t beams, OutputDestination dest,
                                                               uint32_t search_start, uint32_t search_end) {
  uint32_t s = 0, e = 0, cap = 0;
  ctx_->check((spx_status)spx_all_maxima_capacity(params_.nFFT, search_start, search_end, 1000, &s, &e, &cap),
              "FindAllMaxima");
  void *d_out, *d_counts;
  alloc_outputs((uint32_t)beams, cap, &d_out, &d_counts);
  spx_peak_params p{};
  p.mode = SPX_PEAK_ALL;
  p.search_start = search_start;
  p.search_end = search_end;
  p.max_per_beam = 1000;
  p.refine = SPX_REFINE_NONE;
  p.sample_rate = params_.sample_rate;
  spectrum_gb300::StageTimer tm(spx_get_stream(ctx_->get()));
  size_t m0 = tm.mark();
  spx_status st = spx_fft_peaks(ctx_->get(), d_in, (uint32_t)beams, params_.n_point, params_.nFFT, SPX_WINDOW_NONE,
                                &p, static_cast<spx_max_value*>(d_out), static_cast<uint32_t*>(d_counts));
  size_t m1 = tm.mark();
  if (st == SPX_OK) st = spx_synchronize(ctx_->get());
  if (st != SPX_OK) {
    cudaFree(d_out);
    cudaFree(d_counts);
    ctx_->check(st, "FindAllMaxima");
  }
  prof_.fft_time_ms += tm.ms(m0, m1);
  return make_result(*ctx_, d_out, d_counts, (uint32_t)beams, cap, dest);
}

AllMaximaResult SpectrumProcessorGB300::FindAllMaximaFromCPU(const std::vector<std::complex<float>>& data,
                                                             OutputDestination dest, uint32_t search_start,
                                                             uint32_t search_end) {
  if (!initialized_) throw std::runtime_error("SpectrumProcessor::FindAllMaximaFromCPU: not initialized");
  const size_t expected = (size_t)params_.antenna_count * params_.n_point;
  if (data.size() != expected)
    throw std::invalid_argument("FindAllMaximaFromCPU: input size mismatch. Expected " + std::to_string(expected) +
                                ", got " + std::to_string(data.size()));
  if (spectrum_gb300::batch_beams(params_.antenna_count, CalculateBytesPerAntenna(), params_.memory_limit) <
      params_.antenna_count)
    throw std::runtime_error("FindAllMaximaFromCPU: data doesn't fit in GPU memory");
  prof_ = ProfilingData{};
  void* d_in = in_.ensure(expected * 8, "FindAllMaximaFromCPU");
  spectrum_gb300::StageTimer tm(spx_get_stream(ctx_->get()));
  size_t m0 = tm.mark();
  spectrum_gb300::cuda_check(cudaMemcpyAsync(d_in, data.data(), expected * 8, cudaMemcpyHostToDevice, tm.s),
                             "UploadData");
  size_t m1 = tm.mark();
  auto r = all_maxima_from_device(d_in, params_.antenna_count, dest, search_start, search_end);
  prof_.upload_time_ms = tm.ms(m0, m1);
  return r;
}

AllMaximaResult SpectrumProcessorGB300::FindAllMaximaFromGPUPipeline(void* gpu_data, size_t antenna_count,
                                                                     size_t n_point, size_t gpu_memory_bytes,
                                                                     OutputDestination dest, uint32_t search_start,
                                                                     uint32_t search_end) {
  if (!gpu_data) throw std::invalid_argument("FindAllMaximaFromGPUPipeline: gpu_data cannot be null");
  if (!initialized_) throw std::runtime_error("SpectrumProcessor::FindAllMaximaFromGPUPipeline: not initialized");
  if (n_point != params_.n_point)
    throw std::invalid_argument("FindAllMaximaFromGPUPipeline: n_point differs from the initialised n_point");
  if (gpu_memory_bytes && gpu_memory_bytes < antenna_count * n_point * 8)
    throw std::invalid_argument("FindAllMaximaFromGPUPipeline: gpu_memory_bytes too small");
  prof_ = ProfilingData{};
  return all_maxima_from_device(gpu_data, antenna_count, dest, search_start, search_end);
}

// AllMaximaFromCPU (spectrum_processor_rocm.cpp:630-690): spectra already
// computed on the host, uploaded, then the pipeline.
AllMaximaResult SpectrumProcessorGB300::AllMaximaFromCPU(const std::vector<std::complex<float>>& fft_data,
                                                         uint32_t beam_count, uint32_t nFFT, float sample_rate,
                                                         OutputDestination dest, uint32_t search_start,
                                                         uint32_t search_end) {
  const size_t expected = (size_t)beam_count * nFFT;
  if (fft_data.size() != expected)
    throw std::invalid_argument("AllMaximaFromCPU: fft_data size " + std::to_string(fft_data.size()) +
                                " != beam_count * nFFT " + std::to_string(expected));
  void* d = in_.ensure(expected * 8, "AllMaximaFromCPU");
  spectrum_gb300::cuda_check(cudaMemcpyAsync(d, fft_data.data(), expected * 8, cudaMemcpyHostToDevice,
                                             static_cast<cudaStream_t>(spx_get_stream(ctx_->get()))),
                             "AllMaximaFromCPU: H2D");
  return FindAllMaxima(d, beam_count, nFFT, sample_rate, dest, search_start, search_end);
}

// FindAllMaxima (spectrum_processor_rocm.cpp:695-750): window defaults, then
// the pipeline on |X| of the given spectra.
AllMaximaResult SpectrumProcessorGB300::FindAllMaxima(void* fft_data, uint32_t beam_count, uint32_t nFFT,
                                                      float sample_rate, OutputDestination dest,
                                                      uint32_t search_start, uint32_t search_end) {
  if (!fft_data) throw std::invalid_argument("FindAllMaxima: fft_data cannot be null");
  if (search_start == 0) search_start = 1;
  if (search_end == 0) search_end = nFFT / 2;
  if (search_end >= nFFT) search_end = nFFT - 1;
  // the all-maxima stage needs the spectra ordered on this object's stream
  cudaStream_t mine = static_cast<cudaStream_t>(spx_get_stream(ctx_->get()));
  spectrum_gb300::cuda_check(cudaStreamSynchronize(mine), "FindAllMaxima");
  return pipeline_.Execute(nullptr, fft_data, beam_count, nFFT, sample_rate, dest, search_start, search_end);
}

std::unique_ptr<ISpectrumProcessor> SpectrumProcessorFactory::Create(drv_gpu_lib::BackendType backend_type,
                                                                     drv_gpu_lib::IBackend* backend) {
  if (!backend) throw std::invalid_argument("SpectrumProcessorFactory: backend cannot be null");
  switch (backend_type) {
    case drv_gpu_lib::BackendType::AUTO:
    case drv_gpu_lib::BackendType::ROCm:
    case drv_gpu_lib::BackendType::OPENCLandROCm:
    case drv_gpu_lib::BackendType::CUDA:
      return std::make_unique<SpectrumProcessorGB300>(backend);
    case drv_gpu_lib::BackendType::OPENCL:
      throw std::runtime_error("SpectrumProcessorFactory: OpenCL is not supported by this build");
  }
  throw std::invalid_argument("SpectrumProcessorFactory: unknown BackendType");
}

}  // namespace antenna_fft

// ===========================================================================
// spectrum_utils::GpuFFT
// ===========================================================================
namespace spectrum_utils {

namespace {

// One context and staging buffers on device 0 for the static API; never
// destroyed (process-lifetime, like a library singleton).
struct GpuFFTState {
  drv_gpu_lib::CudaBackend backend{0, nullptr};
  spectrum_gb300::Context ctx{&backend};
  spectrum_gb300::DeviceBuffer in, out;
};

GpuFFTState& state() {
  static GpuFFTState* s = new GpuFFTState();
  return *s;
}

template <class In, class Out>
std::vector<Out> run(const std::vector<In>& input, size_t out_len, const char* where,
                     const std::function<spx_status(spx_ctx*, const void*, void*)>& call) {
  if (input.empty()) throw std::runtime_error(std::string("GpuFFT::") + where + ": empty input");
  GpuFFTState& st = state();
  void* d_in = st.in.ensure(input.size() * sizeof(In), where);
  void* d_out = st.out.ensure(out_len * sizeof(Out), where);
  spectrum_gb300::cuda_check(cudaMemcpy(d_in, input.data(), input.size() * sizeof(In), cudaMemcpyHostToDevice), where);
  st.ctx.check(call(st.ctx.get(), d_in, d_out), where);
  st.ctx.check(spx_synchronize(st.ctx.get()), where);
  std::vector<Out> r(out_len);
  spectrum_gb300::cuda_check(cudaMemcpy(r.data(), d_out, out_len * sizeof(Out), cudaMemcpyDeviceToHost), where);
  return r;
}

// The transform size of an input of `len` elements, rejected before any
// device memory is taken when this build has no transform of that length.
uint32_t transform_len(size_t len, const char* where) {
  if (len > 0 && (len > 0xffffffffull || !spx_fft_size_supported((uint32_t)len)))
    throw std::invalid_argument(std::string("GpuFFT::") + where + ": length " + std::to_string(len) +
                                " is not a transform size of this build");
  return (uint32_t)len;
}

}  // namespace

std::vector<std::complex<float>> GpuFFT::ForwardC2C(const std::vector<std::complex<float>>& input) {
  const uint32_t n = transform_len(input.size(), "ForwardC2C");
  return run<std::complex<float>, std::complex<float>>(input, n, "ForwardC2C", [n](spx_ctx* c, const void* i, void* o) {
    return spx_fft(c, i, 1, n, n, SPX_WINDOW_NONE, SPX_OUT_COMPLEX, 1.0f, o);
  });
}

std::vector<std::complex<float>> GpuFFT::InverseC2C(const std::vector<std::complex<float>>& input) {
  const uint32_t n = transform_len(input.size(), "InverseC2C");
  return run<std::complex<float>, std::complex<float>>(input, n, "InverseC2C", [n](spx_ctx* c, const void* i, void* o) {
    return spx_ifft(c, i, 1, n, o);
  });
}

std::vector<std::complex<float>> GpuFFT::ForwardR2C(const std::vector<float>& input) {
  const uint32_t n = transform_len(input.size(), "ForwardR2C");
  return run<float, std::complex<float>>(input, n / 2 + 1, "ForwardR2C", [n](spx_ctx* c, const void* i, void* o) {
    return spx_fft_r2c(c, static_cast<const float*>(i), 1, n, n, SPX_WINDOW_NONE, 0, o);
  });
}

std::vector<std::complex<float>> GpuFFT::ForwardR2C_Full(const std::vector<float>& input) {
  const uint32_t n = transform_len(input.size(), "ForwardR2C_Full");
  return run<float, std::complex<float>>(input, n, "ForwardR2C_Full", [n](spx_ctx* c, const void* i, void* o) {
    return spx_fft_r2c(c, static_cast<const float*>(i), 1, n, n, SPX_WINDOW_NONE, 1, o);
  });
}

std::vector<float> GpuFFT::Magnitude(const std::vector<std::complex<float>>& spectrum, bool squared) {
  if (spectrum.empty()) return {};
  const uint64_t n = spectrum.size();
  return run<std::complex<float>, float>(spectrum, n, "Magnitude", [n, squared](spx_ctx* c, const void* i, void* o) {
    return spx_magnitude(c, i, static_cast<float*>(o), n, 1.0f, squared ? 1 : 0);
  });
}

}  // namespace spectrum_utils
