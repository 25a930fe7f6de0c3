// facade_kat.cpp — known-answer tests of the C++ facades, written against the
// reference's class names (spectrum_gb300/rocm_names.hpp) the way the
// reference's own suites exercise them:
//   tests/test_fft_processor_rocm.hpp        (single_beam_complex, multi_beam_batch,
//                                             mag_phase_consistency, mag_phase_freq, gpu_input)
//   tests/test_complex_to_mag_phase_rocm.hpp (3-4-5 accuracy, gpu paths)
//   tests/test_process_magnitude_rocm.hpp    (norm_coeff handling)
//   tests/test_spectrum_maxima_rocm.hpp      (one_peak, two_peaks, find_all_maxima,
//                                             all_maxima_fft, batch_16_beams)
// plus ownership of GPU results and the exception mapping.
//
// Usage: facade_kat            run everything on device 0 (needs a GPU)
//        facade_kat --no-gpu   only the checks that need no GPU
// Prints one line per check and "SUMMARY <passed> <failed>"; exit code 0 iff
// nothing failed.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
#include <functional>
#include <stdexcept>
#include <string>
#include <vector>

#include "spectrum_gb300/rocm_names.hpp"

using namespace fft_processor;
using namespace antenna_fft;
using drv_gpu_lib::BackendType;
using drv_gpu_lib::CudaBackend;

static int g_pass = 0, g_fail = 0;

static void check(bool ok, const std::string& name, const std::string& detail = "") {
  std::printf("%s %s %s\n", ok ? "PASS" : "FAIL", name.c_str(), detail.c_str());
  (ok ? g_pass : g_fail)++;
}

template <class E>
static void expect_throw(const std::string& name, const std::function<void()>& fn) {
  try {
    fn();
    check(false, name, "no exception");
  } catch (const E&) {
    check(true, name);
  } catch (const std::exception& e) {
    check(false, name, std::string("wrong exception: ") + e.what());
  }
}

static const float kPi = 3.14159265358979323846f;

// complex tone exp(i 2 pi f t / fs) per beam
static std::vector<std::complex<float>> tone(float f, float fs, uint32_t n, uint32_t beams = 1) {
  std::vector<std::complex<float>> x((size_t)beams * n);
  for (uint32_t b = 0; b < beams; ++b)
    for (uint32_t t = 0; t < n; ++t) {
      const double ph = 2.0 * M_PI * (double)f * t / fs;
      x[(size_t)b * n + t] = {(float)std::cos(ph), (float)std::sin(ph)};
    }
  return x;
}

// real sum of sines (the reference's CW generators put the signal in the real part)
static std::vector<std::complex<float>> real_sines(const std::vector<float>& fr, float fs, uint32_t n,
                                                   uint32_t beams) {
  std::vector<std::complex<float>> x((size_t)beams * n);
  for (uint32_t b = 0; b < beams; ++b)
    for (uint32_t t = 0; t < n; ++t) {
      float v = 0.f;
      for (float f : fr) v += std::sin(2.0f * kPi * f * (float)t / fs);
      x[(size_t)b * n + t] = {v, 0.f};
    }
  return x;
}

static size_t peak_bin(const std::vector<float>& m, size_t n) {
  size_t k = 0;
  for (size_t i = 1; i < n; ++i)
    if (m[i] > m[k]) k = i;
  return k;
}

static void fft_tests(CudaBackend& be) {
  {  // single_beam_complex: 100 Hz at fs 1 kHz, 1024 points -> bin 102
    FFTProcessorROCm fft(&be);
    FFTProcessorParams p;
    p.beam_count = 1;
    p.n_point = 1024;
    p.sample_rate = 1000.f;
    auto r = fft.ProcessComplex(tone(100.f, 1000.f, 1024), p);
    std::vector<float> m(r[0].nFFT);
    for (size_t k = 0; k < m.size(); ++k) m[k] = std::abs(r[0].spectrum[k]);
    const size_t pk = peak_bin(m, r[0].nFFT / 2);
    check(r.size() == 1 && r[0].nFFT == 1024 && pk == 102, "fft.single_beam_complex", "peak " + std::to_string(pk));
  }
  {  // multi_beam_batch: 8 beams at 50 + 25 b Hz, peak within one bin
    FFTProcessorROCm fft(&be);
    FFTProcessorParams p;
    p.beam_count = 8;
    p.n_point = 1024;
    p.sample_rate = 1000.f;
    std::vector<std::complex<float>> x;
    for (uint32_t b = 0; b < 8; ++b) {
      auto t = tone(50.f + 25.f * b, 1000.f, 1024);
      x.insert(x.end(), t.begin(), t.end());
    }
    auto r = fft.ProcessComplex(x, p);
    bool ok = r.size() == 8;
    for (uint32_t b = 0; ok && b < 8; ++b) {
      std::vector<float> m(r[b].nFFT);
      for (size_t k = 0; k < m.size(); ++k) m[k] = std::abs(r[b].spectrum[k]);
      const long exp = std::lround((50.f + 25.f * b) * 1024.f / 1000.f);
      const long pk = (long)peak_bin(m, 512);
      ok = ok && std::labs(pk - exp) <= 1 && r[b].beam_id == b;
    }
    check(ok, "fft.multi_beam_batch");
  }
  {  // mag_phase_consistency + mag_phase_freq + repeat_count zero padding
    FFTProcessorROCm fft(&be);
    FFTProcessorParams p;
    p.beam_count = 2;
    p.n_point = 1000;
    p.sample_rate = 1000.f;
    p.repeat_count = 2;
    auto x = tone(150.f, 1000.f, 1000, 2);
    auto cr = fft.ProcessComplex(x, p);
    p.output_mode = FFTOutputMode::MAGNITUDE_PHASE_FREQ;
    auto mr = fft.ProcessMagPhase(x, p);
    const uint32_t n = cr[0].nFFT;
    float me = 0.f, pe = 0.f, fe = 0.f;
    for (uint32_t k = 0; k < n; ++k) {
      const float cm = std::abs(cr[1].spectrum[k]);
      me = std::max(me, std::fabs(cm - mr[1].magnitude[k]) / std::max(1.f, cm));
      float d = std::fabs(std::arg(cr[1].spectrum[k]) - mr[1].phase[k]);
      if (d > kPi) d = 2 * kPi - d;
      if (cm > 1e-3f) pe = std::max(pe, d);
      fe = std::max(fe, std::fabs(mr[1].frequency[k] - (float)k * (1000.f / (float)n)));
    }
    check(n == 2048 && cr.size() == 2 && mr.size() == 2, "fft.repeat_count_nfft", "nFFT " + std::to_string(n));
    check(me < 1e-5f && pe < 1e-5f, "fft.mag_phase_consistency",
          "mag " + std::to_string(me) + " phase " + std::to_string(pe));
    const size_t pk = peak_bin(mr[1].magnitude, n / 2);
    check(fe < 1e-4f && std::fabs(mr[1].frequency[pk] - 150.f) <= 1000.f / n, "fft.mag_phase_freq");
    check(mr[0].frequency.size() == n, "fft.frequency_present");
    p.output_mode = FFTOutputMode::MAGNITUDE_PHASE;
    auto mr2 = fft.ProcessMagPhase(x, p);
    check(mr2[0].frequency.empty(), "fft.frequency_absent_without_freq_mode");
  }
  {  // gpu_input: device pointer path equals the host path bit for bit
    FFTProcessorROCm fft(&be);
    FFTProcessorParams p;
    p.beam_count = 3;
    p.n_point = 4096;
    p.sample_rate = 1.f;
    auto x = tone(0.123f, 1.f, 4096, 3);
    void* d = nullptr;
    cudaMalloc(&d, x.size() * 8);
    cudaMemcpy(d, x.data(), x.size() * 8, cudaMemcpyHostToDevice);
    auto a = fft.ProcessComplex(x, p);
    auto b = fft.ProcessComplex(d, p, x.size() * 8);
    bool same = a.size() == b.size();
    for (size_t i = 0; same && i < a.size(); ++i)
      same = std::memcmp(a[i].spectrum.data(), b[i].spectrum.data(), a[i].spectrum.size() * 8) == 0;
    check(same, "fft.gpu_input_equals_host_input");
    // ProcessMagnitudesToGPU: Hann window, |X|^2 into a caller buffer
    float* dm = nullptr;
    cudaMalloc(&dm, 3 * 4096 * 4);
    fft.ProcessMagnitudesToGPU(d, dm, p, true, WindowType::Hann);
    std::vector<float> m(3 * 4096);
    cudaMemcpy(m.data(), dm, m.size() * 4, cudaMemcpyDeviceToHost);
    const size_t pk = peak_bin(std::vector<float>(m.begin(), m.begin() + 4096), 4096);
    check(std::labs((long)pk - std::lround(0.123 * 4096)) <= 1 && m[pk] > 1e6f, "fft.magnitudes_to_gpu_hann_squared",
          "peak " + std::to_string(pk) + " value " + std::to_string(m[pk]));
    cudaFree(dm);
    cudaFree(d);
    expect_throw<std::invalid_argument>("fft.null_gpu_data", [&] { fft.ProcessComplex(nullptr, p); });
    expect_throw<std::invalid_argument>("fft.gpu_bytes_too_small", [&] { fft.ProcessComplex((void*)16, p, 8); });
  }
  {
    FFTProcessorROCm fft(&be);
    FFTProcessorParams p;
    p.beam_count = 2;
    p.n_point = 100;
    expect_throw<std::invalid_argument>("fft.size_mismatch",
                                        [&] { fft.ProcessComplex(std::vector<std::complex<float>>(199), p); });
    p.n_point = 1 << 20;
    p.repeat_count = 512;  // 2^29: beyond this build's sizes
    expect_throw<std::invalid_argument>("fft.unsupported_nfft",
                                        [&] { fft.ProcessComplex(std::vector<std::complex<float>>(2 << 20), p); });
  }
  {  // nextPow2(2^20) x repeat_count 4 = 2^22 (the four-step transform): a tone at 1000 Hz of fs 2^20 Hz
    FFTProcessorROCm fft(&be);
    FFTProcessorParams p;
    p.beam_count = 1;
    p.n_point = 1 << 20;
    p.sample_rate = (float)(1 << 20);
    p.repeat_count = 4;
    p.output_mode = FFTOutputMode::MAGNITUDE_PHASE;
    auto r = fft.ProcessMagPhase(tone(1000.f, (float)(1 << 20), 1 << 20, 1), p);
    const uint32_t n = r[0].nFFT;
    const size_t pk = peak_bin(r[0].magnitude, n / 2);
    check(n == (1u << 22) && pk == 4000 && std::fabs(r[0].magnitude[pk] - (float)(1 << 20)) < 10.0f,
          "fft.repeat_count_four_step", "nFFT " + std::to_string(n) + " peak " + std::to_string(pk));
  }
}

static void mag_tests(CudaBackend& be) {
  ComplexToMagPhaseROCm c(&be);
  std::vector<std::complex<float>> z = {{3.f, 4.f}, {0.f, 0.f}, {-3.f, -4.f}, {0.f, 1.f}};
  MagPhaseParams p;
  p.beam_count = 2;
  p.n_point = 2;
  auto r = c.Process(z, p);
  check(r.size() == 2 && r[0].magnitude[0] == 5.f && r[0].magnitude[1] == 0.f && r[1].magnitude[0] == 5.f &&
            std::fabs(r[1].phase[1] - kPi / 2) < 1e-6f && r[1].beam_id == 1,
        "mag.accuracy_345");
  void* d = nullptr;
  cudaMalloc(&d, z.size() * 8);
  cudaMemcpy(d, z.data(), z.size() * 8, cudaMemcpyHostToDevice);
  p.norm_coeff = -1.f;  // divide by n_point
  auto m = c.ProcessMagnitude(d, p);
  check(m.size() == 2 && m[0].magnitude[0] == 2.5f && m[1].magnitude[0] == 2.5f, "mag.norm_by_n");
  p.norm_coeff = 0.f;
  m = c.ProcessMagnitude(d, p);
  check(m[0].magnitude[0] == 5.f, "mag.norm_zero_is_one");
  p.norm_coeff = 2.f;
  float* out = static_cast<float*>(c.ProcessMagnitudeToGPU(d, p));
  float h[4];
  cudaMemcpy(h, out, 16, cudaMemcpyDeviceToHost);
  check(h[0] == 10.f && h[3] == 2.f, "mag.to_gpu_caller_owns");
  cudaFree(out);
  float* mp = static_cast<float*>(c.ProcessToGPU(z, p));
  float hp[8];
  cudaMemcpy(hp, mp, 32, cudaMemcpyDeviceToHost);
  check(hp[0] == 5.f && std::fabs(hp[1] - std::atan2(4.f, 3.f)) < 1e-6f, "mag.process_to_gpu_interleaved");
  cudaFree(mp);
  float* buf = nullptr;
  cudaMalloc(&buf, 16);
  p.norm_coeff = 1.f;
  c.ProcessMagnitudeToBuffer(d, buf, p);
  cudaMemcpy(h, buf, 16, cudaMemcpyDeviceToHost);
  check(h[0] == 5.f && h[1] == 0.f, "mag.to_buffer");
  cudaFree(buf);
  cudaFree(d);
  expect_throw<std::invalid_argument>("mag.null", [&] { c.ProcessMagnitude(nullptr, p); });
}

static void spectrum_tests(CudaBackend& be) {
  {  // one_peak: 100 Hz at fs 10 kHz, 1000 points, 4 beams -> within 5 Hz
    auto proc = SpectrumProcessorFactory::Create(BackendType::ROCm, &be);
    SpectrumParams p;
    p.antenna_count = 4;
    p.n_point = 1000;
    p.repeat_count = 1;
    p.sample_rate = 10000.f;
    p.peak_mode = PeakSearchMode::ONE_PEAK;
    expect_throw<std::runtime_error>("spectrum.not_initialized",
                                     [&] { proc->ProcessFromCPU(real_sines({100.f}, 10000.f, 1000, 4)); });
    proc->Initialize(p);
    auto r = proc->ProcessFromCPU(real_sines({100.f}, 10000.f, 1000, 4));
    bool ok = r.size() == 4;
    for (auto& x : r) ok = ok && std::fabs(x.interpolated.refined_frequency - 100.f) < 5.f;
    check(ok, "spectrum.one_peak", r.empty() ? "" : std::to_string(r[0].interpolated.refined_frequency));
    check(r[0].center_point.index == r[0].interpolated.index && r[0].left_point.index + 1 == r[0].center_point.index &&
              r[0].right_point.index == r[0].center_point.index + 1,
          "spectrum.one_peak_neighbours");
    expect_throw<std::invalid_argument>("spectrum.size_mismatch",
                                        [&] { proc->ProcessFromCPU(std::vector<std::complex<float>>(5)); });
  }
  {  // two_peaks: 2 beams -> 4 results
    auto proc = SpectrumProcessorFactory::Create(BackendType::AUTO, &be);
    SpectrumParams p;
    p.antenna_count = 2;
    p.n_point = 1000;
    p.repeat_count = 1;
    p.sample_rate = 10000.f;
    p.peak_mode = PeakSearchMode::TWO_PEAKS;
    proc->Initialize(p);
    auto r = proc->ProcessFromCPU(real_sines({100.f, 300.f}, 10000.f, 1000, 2));
    check(r.size() == 4 && r[0].antenna_id == 0 && r[1].antenna_id == 0 && r[2].antenna_id == 1, "spectrum.two_peaks");
  }
  {  // find_all_maxima: 50 / 120 / 200 Hz at fs 1 kHz -> >= 3 maxima per beam; dest ALL
    auto proc = SpectrumProcessorFactory::Create(BackendType::ROCm, &be);
    SpectrumParams p;
    p.antenna_count = 2;
    p.n_point = 1024;
    p.repeat_count = 1;
    p.sample_rate = 1000.f;
    proc->Initialize(p);
    auto x = real_sines({50.f, 120.f, 200.f}, 1000.f, 1024, 2);
    auto r = proc->FindAllMaximaFromCPU(x, OutputDestination::CPU, 1, 0);
    bool ok = r.total_maxima > 0 && r.beams.size() == 2;
    for (auto& b : r.beams) ok = ok && b.num_maxima >= 3 && b.maxima.size() == b.num_maxima;
    check(ok, "spectrum.find_all_maxima", "total " + std::to_string(r.total_maxima));
    uint32_t s0 = 0, e0 = 0, cap = 0;
    spx_all_maxima_capacity(1024, 1, 0, 1000, &s0, &e0, &cap);  // min((512 - 1) / 2, 1000) = 255
    auto ra = proc->FindAllMaximaFromCPU(x, OutputDestination::ALL, 1, 0);
    bool own = cap == 255 && ra.gpu_maxima && ra.gpu_counts && ra.gpu_bytes == 2 * cap * sizeof(MaxValue) &&
               ra.total_maxima == r.total_maxima;
    std::vector<MaxValue> g(2 * cap);
    uint32_t cnt[2];
    cudaMemcpy(g.data(), ra.gpu_maxima, ra.gpu_bytes, cudaMemcpyDeviceToHost);
    cudaMemcpy(cnt, ra.gpu_counts, 8, cudaMemcpyDeviceToHost);
    for (uint32_t b = 0; own && b < 2; ++b) {
      own = own && std::min(cnt[b], cap) == r.beams[b].num_maxima;
      for (uint32_t i = 0; own && i < r.beams[b].num_maxima; ++i)
        own = g[b * cap + i].index == r.beams[b].maxima[i].index;
    }
    check(own, "spectrum.all_maxima_dest_all_caller_owns");
    cudaFree(ra.gpu_maxima);
    cudaFree(ra.gpu_counts);
    // GPU only: total_maxima sums the untruncated counts
    auto rg = proc->FindAllMaximaFromCPU(x, OutputDestination::GPU, 1, 0);
    check(rg.beams.empty() && rg.gpu_maxima && rg.total_maxima == (size_t)cnt[0] + cnt[1],
          "spectrum.all_maxima_dest_gpu");
    cudaFree(rg.gpu_maxima);
    cudaFree(rg.gpu_counts);
    // the same search on the spectra through FindAllMaxima and through the GPU pipeline
    void* d = nullptr;
    cudaMalloc(&d, x.size() * 8);
    cudaMemcpy(d, x.data(), x.size() * 8, cudaMemcpyHostToDevice);
    auto rp = proc->FindAllMaximaFromGPUPipeline(d, 2, 1024, x.size() * 8, OutputDestination::CPU, 0, 0);
    check(rp.total_maxima == r.total_maxima, "spectrum.from_gpu_pipeline_equals_from_cpu");
    cudaFree(d);
  }
  {  // all_maxima_fft: a 0.1 floor with bins 50 / 120 / 200 -> exactly those three
    auto proc = SpectrumProcessorFactory::Create(BackendType::ROCm, &be);
    SpectrumParams p;
    p.antenna_count = 1;
    p.n_point = 1024;
    p.repeat_count = 1;
    p.sample_rate = 1000.f;
    proc->Initialize(p);
    std::vector<std::complex<float>> f(1024, {0.1f, 0.f});
    f[50] = {100.f, 0.f};
    f[120] = {80.f, 0.f};
    f[200] = {60.f, 0.f};
    auto r = proc->AllMaximaFromCPU(f, 1, 1024, 1000.f, OutputDestination::CPU, 1, 512);
    bool ok = r.total_maxima == 3 && r.beams[0].maxima[0].index == 50 && r.beams[0].maxima[1].index == 120 &&
              r.beams[0].maxima[2].index == 200 && r.beams[0].maxima[0].magnitude == 100.f &&
              std::fabs(r.beams[0].maxima[1].refined_frequency - 120.f * 1000.f / 1024.f) < 1e-3f;
    check(ok, "spectrum.all_maxima_fft", "total " + std::to_string(r.total_maxima));
    // the pipeline itself, magnitudes supplied by ComplexToMagPhase
    AllMaximaPipelineROCm pipe(&be);
    void* d = nullptr;
    cudaMalloc(&d, f.size() * 8);
    cudaMemcpy(d, f.data(), f.size() * 8, cudaMemcpyHostToDevice);
    ComplexToMagPhaseROCm c(&be);
    MagPhaseParams mp;
    mp.beam_count = 1;
    mp.n_point = 1024;
    void* mag = c.ProcessMagnitudeToGPU(d, mp);
    auto rp = pipe.Execute(mag, d, 1, 1024, 1000.f);
    check(rp.total_maxima == 3 && rp.beams[0].maxima[2].index == 200, "pipeline.execute_with_magnitudes");
    cudaFree(mag);
    cudaFree(d);
  }
  {  // batch_16_beams: 100 + 10 b Hz at fs 10 kHz -> within 10 Hz
    auto proc = SpectrumProcessorFactory::Create(BackendType::ROCm, &be);
    SpectrumParams p;
    p.antenna_count = 16;
    p.n_point = 1000;
    p.repeat_count = 1;
    p.sample_rate = 10000.f;
    proc->Initialize(p);
    std::vector<std::complex<float>> x;
    for (uint32_t b = 0; b < 16; ++b) {
      auto s = real_sines({100.f + 10.f * b}, 10000.f, 1000, 1);
      x.insert(x.end(), s.begin(), s.end());
    }
    auto r = proc->ProcessFromCPU(x);
    bool ok = r.size() == 16;
    for (auto& y : r) ok = ok && std::fabs(y.interpolated.refined_frequency - (100.f + 10.f * y.antenna_id)) < 10.f;
    check(ok, "spectrum.batch_16_beams");
  }
  expect_throw<std::runtime_error>("factory.opencl_rejected",
                                   [&] { SpectrumProcessorFactory::Create(BackendType::OPENCL, &be); });
  expect_throw<std::invalid_argument>("factory.null_backend",
                                      [&] { SpectrumProcessorFactory::Create(BackendType::ROCm, nullptr); });
}

static void gpufft_tests() {
  using spectrum_utils::GpuFFT;
  // forward against a direct DFT (n = 96), inverse round trip, R2C half / full
  const uint32_t n = 96;
  std::vector<std::complex<float>> x(n);
  std::vector<float> r(n);
  for (uint32_t t = 0; t < n; ++t) {
    x[t] = {std::cos(0.3f * t) + 0.1f * t / n, std::sin(0.7f * t)};
    r[t] = std::cos(0.25f * t) - 0.5f * std::sin(0.9f * t);
  }
  auto X = GpuFFT::ForwardC2C(x);
  double err = 0.0, peak = 0.0;
  for (uint32_t k = 0; k < n; ++k) {
    std::complex<double> acc = 0.0;
    for (uint32_t t = 0; t < n; ++t) acc += std::complex<double>(x[t]) * std::polar(1.0, -2.0 * M_PI * k * t / n);
    err = std::max(err, std::abs(acc - std::complex<double>(X[k])));
    peak = std::max(peak, std::abs(acc));
  }
  check(X.size() == n && err / peak < 1e-5, "gpufft.forward_c2c_vs_dft", std::to_string(err / peak));
  auto back = GpuFFT::InverseC2C(X);
  double rt = 0.0;
  for (uint32_t t = 0; t < n; ++t) rt = std::max(rt, (double)std::abs(back[t] - x[t]));
  check(rt < 1e-5, "gpufft.inverse_round_trip", std::to_string(rt));
  auto half = GpuFFT::ForwardR2C(r);
  auto full = GpuFFT::ForwardR2C_Full(r);
  bool mirror = half.size() == n / 2 + 1 && full.size() == n;
  for (uint32_t k = 0; mirror && k <= n / 2; ++k) mirror = full[k] == half[k];
  for (uint32_t k = n / 2 + 1; mirror && k < n; ++k) mirror = full[k] == std::conj(full[n - k]);
  check(mirror, "gpufft.r2c_half_and_full_mirror");
  auto m = GpuFFT::Magnitude({{3.f, 4.f}, {0.f, 0.f}}, false);
  auto m2 = GpuFFT::Magnitude({{3.f, 4.f}}, true);
  check(m.size() == 2 && m[0] == 5.f && m[1] == 0.f && m2[0] == 25.f, "gpufft.magnitude");
  expect_throw<std::runtime_error>("gpufft.empty", [] { GpuFFT::ForwardC2C({}); });
  {  // CpuFFT takes any length: 1000 = 2^3 5^3 (Bluestein's transform on the GPU)
    const uint32_t n1 = 1000;
    std::vector<std::complex<float>> y(n1);
    for (uint32_t t = 0; t < n1; ++t) y[t] = {std::cos(0.11f * t), std::sin(0.37f * t) + 0.2f};
    auto Y = GpuFFT::ForwardC2C(y);
    double e1 = 0.0, p1 = 0.0;
    for (uint32_t k = 0; k < n1; ++k) {
      std::complex<double> acc = 0.0;
      for (uint32_t t = 0; t < n1; ++t) acc += std::complex<double>(y[t]) * std::polar(1.0, -2.0 * M_PI * k * t / n1);
      e1 = std::max(e1, std::abs(acc - std::complex<double>(Y[k])));
      p1 = std::max(p1, std::abs(acc));
    }
    check(Y.size() == n1 && e1 / p1 < 1e-5, "gpufft.any_length_1000", std::to_string(e1 / p1));
  }
  expect_throw<std::invalid_argument>("gpufft.unsupported_length", [] {
    GpuFFT::ForwardC2C(std::vector<std::complex<float>>((1u << 27) + 1));  // too long for Bluestein's transform
  });
}

int main(int argc, char** argv) {
  const bool no_gpu = argc > 1 && std::strcmp(argv[1], "--no-gpu") == 0;
  if (no_gpu) {
    // without a device every facade refuses to construct with std::runtime_error
    CudaBackend be(0);
    expect_throw<std::runtime_error>("nogpu.fft_processor", [&] { FFTProcessorROCm f(&be); });
    expect_throw<std::runtime_error>("nogpu.spectrum_processor",
                                     [&] { SpectrumProcessorFactory::Create(BackendType::ROCm, &be); });
    expect_throw<std::invalid_argument>("nogpu.null_backend", [&] { FFTProcessorROCm f(nullptr); });
  } else {
    cudaStream_t s;
    cudaStreamCreate(&s);
    CudaBackend be(0, s);
    try {
      fft_tests(be);
      mag_tests(be);
      spectrum_tests(be);
      gpufft_tests();
    } catch (const std::exception& e) {
      check(false, "unexpected exception", e.what());
    }
    cudaStreamDestroy(s);
  }
  std::printf("SUMMARY %d %d\n", g_pass, g_fail);
  return g_fail == 0 ? 0 : 1;
}
