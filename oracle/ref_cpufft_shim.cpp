// ref_cpufft_shim.cpp — extern "C" access to the reference's CPU FFT
// (spectrum_utils::CpuFFT, include/spectrum/utils/cpu_fft.hpp:68-203, which
// wraps its vendored pocketfft).  TEST INFRASTRUCTURE ONLY: compiled by
// oracle/build_ref.py against the reference's headers into oracle/_ref/.
#include <complex>
#include <cstddef>
#include <vector>

#include <spectrum/utils/cpu_fft.hpp>

extern "C" {

// Forward C2C of `beams` rows of n complex64 values (interleaved floats).
int ref_cpu_fft_c2c(const float* in, float* out, size_t beams, size_t n) {
  std::vector<std::complex<float>> v(n);
  for (size_t b = 0; b < beams; ++b) {
    const float* x = in + 2 * b * n;
    for (size_t i = 0; i < n; ++i) v[i] = {x[2 * i], x[2 * i + 1]};
    auto r = spectrum_utils::CpuFFT::ForwardC2C(v);
    float* y = out + 2 * b * n;
    for (size_t i = 0; i < n; ++i) {
      y[2 * i] = r[i].real();
      y[2 * i + 1] = r[i].imag();
    }
  }
  return 0;
}

// CpuFFT::InverseC2C (1/N) of `beams` rows of n complex64 values.
int ref_cpu_ifft_c2c(const float* in, float* out, size_t beams, size_t n) {
  std::vector<std::complex<float>> v(n);
  for (size_t b = 0; b < beams; ++b) {
    const float* x = in + 2 * b * n;
    for (size_t i = 0; i < n; ++i) v[i] = {x[2 * i], x[2 * i + 1]};
    auto r = spectrum_utils::CpuFFT::InverseC2C(v);
    float* y = out + 2 * b * n;
    for (size_t i = 0; i < n; ++i) {
      y[2 * i] = r[i].real();
      y[2 * i + 1] = r[i].imag();
    }
  }
  return 0;
}

// CpuFFT::ForwardR2C (full = 0: n/2 + 1 bins) or ForwardR2C_Full (full = 1:
// n bins) of `beams` rows of n floats.
int ref_cpu_fft_r2c(const float* in, float* out, size_t beams, size_t n, int full) {
  std::vector<float> v(n);
  const size_t m = full ? n : n / 2 + 1;
  for (size_t b = 0; b < beams; ++b) {
    for (size_t i = 0; i < n; ++i) v[i] = in[b * n + i];
    auto r = full ? spectrum_utils::CpuFFT::ForwardR2C_Full(v) : spectrum_utils::CpuFFT::ForwardR2C(v);
    float* y = out + 2 * b * m;
    for (size_t i = 0; i < m; ++i) {
      y[2 * i] = r[i].real();
      y[2 * i + 1] = r[i].imag();
    }
  }
  return 0;
}

// CpuFFT::Magnitude: |X| or |X|^2.
int ref_cpu_magnitude(const float* in, float* out, size_t n, int squared) {
  std::vector<std::complex<float>> v(n);
  for (size_t i = 0; i < n; ++i) v[i] = {in[2 * i], in[2 * i + 1]};
  auto m = spectrum_utils::CpuFFT::Magnitude(v, squared != 0);
  for (size_t i = 0; i < n; ++i) out[i] = m[i];
  return 0;
}

}  // extern "C"
