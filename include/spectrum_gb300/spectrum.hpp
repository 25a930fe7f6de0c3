// spectrum.hpp — C++ facades of the GB300 FFT -> |X| -> peaks path.
//
// The classes keep the reference's (DspSpectrum) class shapes, method names,
// argument meaning, result types and exceptions, and run everything through
// the C ABI of spx.h:
//   fft_processor::FFTProcessorGB300       <- FFTProcessorROCm
//                                             (include/spectrum/fft_processor_rocm.hpp:53-211)
//   fft_processor::ComplexToMagPhaseGB300  <- ComplexToMagPhaseROCm
//                                             (include/spectrum/complex_to_mag_phase_rocm.hpp:83-270)
//   antenna_fft::ISpectrumProcessor,       <- the same interface
//   antenna_fft::SpectrumProcessorGB300,      (include/spectrum/interface/i_spectrum_processor.hpp:65-170),
//   antenna_fft::SpectrumProcessorFactory     SpectrumProcessorROCm and its factory
//                                             (src/fft_func/src/spectrum_processor_factory.cpp:13-37)
//   antenna_fft::IAllMaximaPipeline,       <- the same interface
//   antenna_fft::AllMaximaPipelineGB300       (include/spectrum/interface/i_all_maxima_pipeline.hpp:55-81)
//   spectrum_utils::GpuFFT                 <- CpuFFT's static API on the GPU
//                                             (include/spectrum/utils/cpu_fft.hpp:68-203)
// spectrum_gb300/rocm_names.hpp adds the reference's *ROCm class names as aliases.
//
// Errors: std::invalid_argument for bad arguments (null pointers, size
// mismatches, sizes this build does not transform); std::runtime_error for
// device failures, as the reference throws.
// Device memory returned to the caller (AllMaximaResult::gpu_maxima /
// gpu_counts with OutputDestination::GPU or ALL, the pointers returned by
// ProcessToGPU / ProcessMagnitudeToGPU) comes from cudaMalloc: release it with
// cudaFree.  Not thread-safe: one object per owning thread, as in the reference.
#pragma once

#include <complex>
#include <cstddef>
#include <cstdint>
#include <memory>
#include <string>
#include <utility>
#include <vector>

#include "spx.h"

// ---------------------------------------------------------------------------
// Runtime shim: device + stream (the part of the reference's DspCore runtime
// the facades use).
// ---------------------------------------------------------------------------
namespace drv_gpu_lib {

enum class OutputDestination { CPU, GPU, ALL };
enum class BackendType { AUTO, OPENCL, ROCm, OPENCLandROCm, CUDA };
enum class DriverType { OPENCL, ROCm, CUDA };

class IBackend {
 public:
  virtual ~IBackend() = default;
  virtual int GetDeviceIndex() const = 0;
  // cudaStream_t the facades order their work on (nullptr = legacy default stream).
  virtual void* GetNativeStream() const = 0;
};

// One CUDA device and a stream the caller owns (or the default stream).
class CudaBackend final : public IBackend {
 public:
  explicit CudaBackend(int device = 0, void* stream = nullptr) : device_(device), stream_(stream) {}
  int GetDeviceIndex() const override { return device_; }
  void* GetNativeStream() const override { return stream_; }

 private:
  int device_;
  void* stream_;
};

// Elapsed time of one stage of a call (CUDA events on the facade's stream).
struct ROCmProfilingData {
  double elapsed_ms = 0.0;
  std::string what;
};

}  // namespace drv_gpu_lib

namespace spectrum_gb300 {

// Owns one spx_ctx bound to a backend's device and stream.
class Context {
 public:
  explicit Context(drv_gpu_lib::IBackend* backend);
  ~Context();
  Context(const Context&) = delete;
  Context& operator=(const Context&) = delete;
  spx_ctx* get() const { return ctx_; }
  int device() const { return device_; }
  // Throws the reference's exception type for a failed spx_* call.
  void check(spx_status st, const char* where) const;

 private:
  spx_ctx* ctx_ = nullptr;
  int device_ = 0;
};

// Grow-only device buffer.
class DeviceBuffer {
 public:
  DeviceBuffer() = default;
  ~DeviceBuffer();
  DeviceBuffer(const DeviceBuffer&) = delete;
  DeviceBuffer& operator=(const DeviceBuffer&) = delete;
  void* ensure(size_t bytes, const char* where);
  void* get() const { return ptr_; }

 private:
  void* ptr_ = nullptr;
  size_t bytes_ = 0;
};

}  // namespace spectrum_gb300

// ---------------------------------------------------------------------------
// FFT processor
// ---------------------------------------------------------------------------
namespace fft_processor {

enum class FFTOutputMode { COMPLEX, MAGNITUDE_PHASE, MAGNITUDE_PHASE_FREQ };

// Window values: NONE..BLACKMAN as the reference; BLACKMAN_HARRIS is this build's extension.
enum class WindowType : uint32_t { None = 0, Hann = 1, Hamming = 2, Blackman = 3, BlackmanHarris = 4 };

struct FFTProcessorParams {
  uint32_t beam_count = 1;
  uint32_t n_point = 0;
  float sample_rate = 1000.0f;
  FFTOutputMode output_mode = FFTOutputMode::COMPLEX;
  uint32_t repeat_count = 1;   // nFFT = nextPow2(n_point) * repeat_count
  float memory_limit = 0.80f;  // fraction of free device memory one batch may use
};

struct FFTBeamResult {
  uint32_t beam_id = 0;
  uint32_t nFFT = 0;
  float sample_rate = 0.0f;
};
struct FFTComplexResult : FFTBeamResult {
  std::vector<std::complex<float>> spectrum;
};
struct FFTMagPhaseResult : FFTBeamResult {
  std::vector<float> magnitude;
  std::vector<float> phase;      // radians
  std::vector<float> frequency;  // k * sample_rate / nFFT (MAGNITUDE_PHASE_FREQ only)
};
struct FFTProfilingData {
  double upload_time_ms = 0.0;
  double fft_time_ms = 0.0;
  double post_processing_time_ms = 0.0;
  double download_time_ms = 0.0;
  double total_time_ms = 0.0;
};

struct MagPhaseParams {
  uint32_t beam_count = 1;
  uint32_t n_point = 0;
  float memory_limit = 0.80f;
  float norm_coeff = 1.0f;  // 0: x1, < 0: x 1/n_point, > 0: x norm_coeff (magnitude only)
};
struct MagPhaseResult {
  uint32_t beam_id = 0;
  uint32_t n_point = 0;
  std::vector<float> magnitude;
  std::vector<float> phase;
};
struct MagnitudeResult {
  uint32_t beam_id = 0;
  uint32_t n_point = 0;
  std::vector<float> magnitude;
};

using ROCmProfEvents = std::vector<std::pair<const char*, drv_gpu_lib::ROCmProfilingData>>;

class FFTProcessorGB300 {
 public:
  explicit FFTProcessorGB300(drv_gpu_lib::IBackend* backend);
  ~FFTProcessorGB300();
  FFTProcessorGB300(const FFTProcessorGB300&) = delete;
  FFTProcessorGB300& operator=(const FFTProcessorGB300&) = delete;
  FFTProcessorGB300(FFTProcessorGB300&&) noexcept;
  FFTProcessorGB300& operator=(FFTProcessorGB300&&) noexcept;

  std::vector<FFTComplexResult> ProcessComplex(const std::vector<std::complex<float>>& data,
                                               const FFTProcessorParams& params,
                                               ROCmProfEvents* prof_events = nullptr);
  std::vector<FFTComplexResult> ProcessComplex(void* gpu_data, const FFTProcessorParams& params,
                                               size_t gpu_memory_bytes = 0);
  std::vector<FFTMagPhaseResult> ProcessMagPhase(const std::vector<std::complex<float>>& data,
                                                 const FFTProcessorParams& params,
                                                 ROCmProfEvents* prof_events = nullptr);
  std::vector<FFTMagPhaseResult> ProcessMagPhase(void* gpu_data, const FFTProcessorParams& params,
                                                 size_t gpu_memory_bytes = 0);
  // |X| (or |X|^2) of the windowed, zero-padded FFT into a caller buffer of
  // beam_count x nFFT floats; no normalisation.
  void ProcessMagnitudesToGPU(void* gpu_data, void* gpu_out_magnitudes, const FFTProcessorParams& params,
                              bool squared = false, WindowType window = WindowType::None,
                              ROCmProfEvents* prof_events = nullptr);
  FFTProfilingData GetProfilingData() const { return prof_; }
  uint32_t GetNFFT() const { return nFFT_; }

 private:
  struct Impl;
  template <class R>
  std::vector<R> run(const std::complex<float>* host, void* gpu, const FFTProcessorParams& params,
                     ROCmProfEvents* prof_events);
  std::unique_ptr<Impl> impl_;
  FFTProfilingData prof_;
  uint32_t nFFT_ = 0;
};

class ComplexToMagPhaseGB300 {
 public:
  explicit ComplexToMagPhaseGB300(drv_gpu_lib::IBackend* backend);
  ~ComplexToMagPhaseGB300();
  ComplexToMagPhaseGB300(const ComplexToMagPhaseGB300&) = delete;
  ComplexToMagPhaseGB300& operator=(const ComplexToMagPhaseGB300&) = delete;
  ComplexToMagPhaseGB300(ComplexToMagPhaseGB300&&) noexcept;
  ComplexToMagPhaseGB300& operator=(ComplexToMagPhaseGB300&&) noexcept;

  std::vector<MagPhaseResult> Process(const std::vector<std::complex<float>>& data, const MagPhaseParams& params);
  std::vector<MagPhaseResult> Process(void* gpu_data, const MagPhaseParams& params, size_t gpu_memory_bytes = 0);
  // Interleaved {|z|, arg z} float pairs in a new device buffer (caller frees with cudaFree).
  void* ProcessToGPU(const std::vector<std::complex<float>>& data, const MagPhaseParams& params);
  void* ProcessToGPU(void* gpu_data, const MagPhaseParams& params, size_t gpu_memory_bytes = 0);
  std::vector<MagnitudeResult> ProcessMagnitude(void* gpu_data, const MagPhaseParams& params,
                                                size_t gpu_memory_bytes = 0);
  // |z| * inv_n in a new device buffer (caller frees with cudaFree).
  void* ProcessMagnitudeToGPU(void* gpu_data, const MagPhaseParams& params, size_t gpu_memory_bytes = 0);
  void ProcessMagnitudeToBuffer(void* gpu_complex_in, void* gpu_magnitude_out, const MagPhaseParams& params);

  // inv_n from norm_coeff (complex_to_mag_phase_rocm.cpp:170-176).
  static float ComputeInvN(const MagPhaseParams& params);

 private:
  struct Impl;
  std::unique_ptr<Impl> impl_;
};

}  // namespace fft_processor

// ---------------------------------------------------------------------------
// Spectrum maxima
// ---------------------------------------------------------------------------
namespace antenna_fft {

using drv_gpu_lib::OutputDestination;

enum class PeakSearchMode { ONE_PEAK, TWO_PEAKS, ALL_MAXIMA };

struct SpectrumParams {
  uint32_t antenna_count = 5;
  uint32_t n_point = 1000;
  uint32_t repeat_count = 2;
  float sample_rate = 1000.0f;
  uint32_t search_range = 0;  // 0 -> nFFT / 4
  PeakSearchMode peak_mode = PeakSearchMode::ONE_PEAK;
  float memory_limit = 0.80f;
  size_t max_maxima_per_beam = 1000;
  uint32_t nFFT = 0;      // computed: nextPow2(n_point) * repeat_count
  uint32_t base_fft = 0;  // computed: nextPow2(n_point)
};

struct MaxValue {
  uint32_t index;
  float real, imag;
  float magnitude;
  float phase;  // degrees
  float freq_offset;
  float refined_frequency;
  uint32_t pad;
};
static_assert(sizeof(MaxValue) == sizeof(spx_max_value), "MaxValue is 32 bytes");

struct SpectrumResult {
  uint32_t antenna_id;
  MaxValue interpolated;
  MaxValue left_point;
  MaxValue center_point;
  MaxValue right_point;
};

struct AllMaximaBeamResult {
  uint32_t antenna_id;
  uint32_t num_maxima;
  std::vector<MaxValue> maxima;
};

struct AllMaximaResult {
  std::vector<AllMaximaBeamResult> beams;
  OutputDestination destination = OutputDestination::CPU;
  void* gpu_maxima = nullptr;  // caller owns (cudaFree) with GPU / ALL
  void* gpu_counts = nullptr;  // caller owns (cudaFree) with GPU / ALL
  size_t total_maxima = 0;
  size_t gpu_bytes = 0;
  size_t TotalMaxima() const { return total_maxima; }
};

struct ProfilingData {
  double upload_time_ms = 0.0;
  double fft_time_ms = 0.0;
  double post_kernel_time_ms = 0.0;
  double download_time_ms = 0.0;
  double total_time_ms = 0.0;
};

class IAllMaximaPipeline {
 public:
  virtual ~IAllMaximaPipeline() = default;
  virtual AllMaximaResult Execute(void* magnitudes_gpu, void* fft_data_gpu, uint32_t beam_count, uint32_t nFFT,
                                  float sample_rate, OutputDestination dest = OutputDestination::CPU,
                                  uint32_t search_start = 1, uint32_t search_end = 0,
                                  size_t max_maxima_per_beam = 1000) = 0;
};

// detect -> compact (one kernel with a decoupled look-back scan) on a
// magnitude array (may be null: |X| is taken from fft_data_gpu).
class AllMaximaPipelineGB300 final : public IAllMaximaPipeline {
 public:
  explicit AllMaximaPipelineGB300(drv_gpu_lib::IBackend* backend);
  ~AllMaximaPipelineGB300() override;
  AllMaximaResult Execute(void* magnitudes_gpu, void* fft_data_gpu, uint32_t beam_count, uint32_t nFFT,
                          float sample_rate, OutputDestination dest = OutputDestination::CPU,
                          uint32_t search_start = 1, uint32_t search_end = 0,
                          size_t max_maxima_per_beam = 1000) override;

 private:
  std::unique_ptr<spectrum_gb300::Context> ctx_;
};

class ISpectrumProcessor {
 public:
  virtual ~ISpectrumProcessor() = default;
  virtual void Initialize(const SpectrumParams& params) = 0;
  virtual bool IsInitialized() const = 0;
  virtual std::vector<SpectrumResult> ProcessFromCPU(const std::vector<std::complex<float>>& data) = 0;
  virtual std::vector<SpectrumResult> ProcessFromGPU(void* gpu_data, size_t antenna_count, size_t n_point,
                                                     size_t gpu_memory_bytes = 0) = 0;
  virtual std::vector<SpectrumResult> ProcessBatch(const std::vector<std::complex<float>>& batch_data,
                                                   size_t start_antenna, size_t batch_antenna_count) = 0;
  virtual std::vector<SpectrumResult> ProcessBatchFromGPU(void* gpu_data, size_t src_offset_bytes,
                                                          size_t start_antenna, size_t batch_antenna_count) = 0;
  virtual AllMaximaResult FindAllMaximaFromCPU(const std::vector<std::complex<float>>& data, OutputDestination dest,
                                               uint32_t search_start, uint32_t search_end) = 0;
  virtual AllMaximaResult FindAllMaximaFromGPUPipeline(void* gpu_data, size_t antenna_count, size_t n_point,
                                                       size_t gpu_memory_bytes, OutputDestination dest,
                                                       uint32_t search_start, uint32_t search_end) = 0;
  virtual AllMaximaResult AllMaximaFromCPU(const std::vector<std::complex<float>>& fft_data, uint32_t beam_count,
                                           uint32_t nFFT, float sample_rate, OutputDestination dest,
                                           uint32_t search_start, uint32_t search_end) = 0;
  virtual AllMaximaResult FindAllMaxima(void* fft_data, uint32_t beam_count, uint32_t nFFT, float sample_rate,
                                        OutputDestination dest = OutputDestination::CPU, uint32_t search_start = 0,
                                        uint32_t search_end = 0) = 0;
  virtual drv_gpu_lib::DriverType GetDriverType() const = 0;
  virtual ProfilingData GetProfilingData() const = 0;
  virtual void ReallocateBuffersForBatch(size_t batch_antenna_count) = 0;
  virtual size_t CalculateBytesPerAntenna() const = 0;
  virtual void CompilePostKernel() = 0;
};

class SpectrumProcessorGB300 final : public ISpectrumProcessor {
 public:
  explicit SpectrumProcessorGB300(drv_gpu_lib::IBackend* backend);
  ~SpectrumProcessorGB300() override;
  SpectrumProcessorGB300(const SpectrumProcessorGB300&) = delete;
  SpectrumProcessorGB300& operator=(const SpectrumProcessorGB300&) = delete;

  void Initialize(const SpectrumParams& params) override;
  bool IsInitialized() const override { return initialized_; }
  std::vector<SpectrumResult> ProcessFromCPU(const std::vector<std::complex<float>>& data) override;
  std::vector<SpectrumResult> ProcessFromGPU(void* gpu_data, size_t antenna_count, size_t n_point,
                                             size_t gpu_memory_bytes = 0) override;
  std::vector<SpectrumResult> ProcessBatch(const std::vector<std::complex<float>>& batch_data, size_t start_antenna,
                                           size_t batch_antenna_count) override;
  std::vector<SpectrumResult> ProcessBatchFromGPU(void* gpu_data, size_t src_offset_bytes, size_t start_antenna,
                                                  size_t batch_antenna_count) override;
  AllMaximaResult FindAllMaximaFromCPU(const std::vector<std::complex<float>>& data, OutputDestination dest,
                                       uint32_t search_start, uint32_t search_end) override;
  AllMaximaResult FindAllMaximaFromGPUPipeline(void* gpu_data, size_t antenna_count, size_t n_point,
                                               size_t gpu_memory_bytes, OutputDestination dest,
                                               uint32_t search_start, uint32_t search_end) override;
  AllMaximaResult AllMaximaFromCPU(const std::vector<std::complex<float>>& fft_data, uint32_t beam_count,
                                   uint32_t nFFT, float sample_rate, OutputDestination dest, uint32_t search_start,
                                   uint32_t search_end) override;
  AllMaximaResult FindAllMaxima(void* fft_data, uint32_t beam_count, uint32_t nFFT, float sample_rate,
                                OutputDestination dest = OutputDestination::CPU, uint32_t search_start = 0,
                                uint32_t search_end = 0) override;
  drv_gpu_lib::DriverType GetDriverType() const override { return drv_gpu_lib::DriverType::CUDA; }
  ProfilingData GetProfilingData() const override { return prof_; }
  void ReallocateBuffersForBatch(size_t batch_antenna_count) override;
  size_t CalculateBytesPerAntenna() const override;
  void CompilePostKernel() override {}  // kernels are compiled ahead of time for sm_103a

  const SpectrumParams& GetParams() const { return params_; }

 private:
  std::vector<SpectrumResult> peaks_from_device(const void* d_in, size_t beams, size_t start_antenna);
  AllMaximaResult all_maxima_from_device(const void* d_in, size_t beams, OutputDestination dest,
                                         uint32_t search_start, uint32_t search_end);
  std::unique_ptr<spectrum_gb300::Context> ctx_;
  spectrum_gb300::DeviceBuffer in_, out_;
  AllMaximaPipelineGB300 pipeline_;
  SpectrumParams params_;
  ProfilingData prof_;
  bool initialized_ = false;
};

class SpectrumProcessorFactory {
 public:
  // AUTO / ROCm / OPENCLandROCm / CUDA -> SpectrumProcessorGB300; OPENCL -> std::runtime_error.
  static std::unique_ptr<ISpectrumProcessor> Create(drv_gpu_lib::BackendType backend_type,
                                                    drv_gpu_lib::IBackend* backend);
};

}  // namespace antenna_fft

// ---------------------------------------------------------------------------
// CpuFFT's static API (include/spectrum/utils/cpu_fft.hpp:68-203) computed on
// GPU 0: host vectors in and out, one transform per call.  Any length from
// 2 to 2^27 (2^a 3^b lengths by the Stockham and four-step plans, others by
// Bluestein's chirp-z transform), and 2^a 3^b lengths up to 2^28 that split
// into two factors <= 16384: std::invalid_argument otherwise; an empty input
// throws std::runtime_error as CpuFFT does.
// ---------------------------------------------------------------------------
namespace spectrum_utils {

struct GpuFFT {
  static std::vector<std::complex<float>> ForwardC2C(const std::vector<std::complex<float>>& input);
  static std::vector<std::complex<float>> InverseC2C(const std::vector<std::complex<float>>& input);
  static std::vector<std::complex<float>> ForwardR2C(const std::vector<float>& input);
  static std::vector<std::complex<float>> ForwardR2C_Full(const std::vector<float>& input);
  static std::vector<float> Magnitude(const std::vector<std::complex<float>>& spectrum, bool squared = false);
};

}  // namespace spectrum_utils
