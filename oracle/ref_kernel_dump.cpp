// ref_kernel_dump.cpp — writes the reference's kernel source strings to files
// (TEST INFRASTRUCTURE ONLY; run by oracle/build_ref.py, outputs go to oracle/_ref/).
// Compiled with -DENABLE_ROCM=1 against the reference's include/ directory.
#include <cstdio>

#include <spectrum/kernels/all_maxima_kernel_sources_rocm.hpp>
#include <spectrum/kernels/fft_kernel_sources_rocm.hpp>
#include <spectrum/kernels/fft_processor_kernels_rocm.hpp>

static int dump(const char* path, const char* text) {
  FILE* f = std::fopen(path, "w");
  if (!f) return 1;
  std::fputs(text, f);
  std::fclose(f);
  return 0;
}

int main(int argc, char** argv) {
  if (argc != 4) {
    std::fprintf(stderr, "usage: %s spectrum.txt allmax.txt fftproc.txt\n", argv[0]);
    return 2;
  }
  int rc = dump(argv[1], antenna_fft::kernels::GetSpectrumHIPKernelSource());
  rc |= dump(argv[2], antenna_fft::kernels::GetAllMaximaHIPKernelSource());
  rc |= dump(argv[3], fft_processor::kernels::GetHIPKernelSource());
  return rc;
}
