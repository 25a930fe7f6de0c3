// ref_kernels_host.cpp — runs the reference's peak-search and magnitude
// kernels on the CPU (TEST INFRASTRUCTURE ONLY, for pinning the oracle).
//
// The kernel bodies are NOT in this repository: oracle/build_ref.py extracts
// them at build time from the reference headers
//   include/spectrum/kernels/fft_kernel_sources_rocm.hpp   (GetSpectrumHIPKernelSource)
//   include/spectrum/kernels/all_maxima_kernel_sources_rocm.hpp (GetAllMaximaHIPKernelSource)
//   include/spectrum/kernels/fft_processor_kernels_rocm.hpp (GetHIPKernelSource)
// into oracle/_ref/gen_*.inc (git-ignored) and compiles this file against
// them.  The extern "C" functions below drive those kernels the way the
// reference's host code does (grids, block sizes, the recursive scan of
// AllMaximaPipelineROCm::ExecutePrefixSum).
#include <ucontext.h>

#include <algorithm>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "ref_simt.h"

ref_uint3 threadIdx{0, 0, 0}, blockIdx{0, 0, 0}, blockDim{1, 1, 1}, gridDim{1, 1, 1};

namespace {

struct Fiber {
  ucontext_t ctx;
  std::vector<char> stack;
  bool done = false;
  ref_uint3 tid{0, 0, 0};
};

ucontext_t g_sched;
std::vector<Fiber> g_fibers;
int g_cur = -1;
const std::function<void()>* g_body = nullptr;
std::vector<unsigned char> g_dyn;
constexpr size_t kStack = 256 * 1024;

void trampoline() {
  const int me = g_cur;
  (*g_body)();
  g_fibers[me].done = true;
  // returning resumes uc_link (the scheduler)
}

void run_block(ref_uint3 block) {
  const unsigned n = block.x * block.y * block.z;
  if (g_fibers.size() < n) g_fibers.resize(n);
  for (unsigned i = 0; i < n; ++i) {
    Fiber& f = g_fibers[i];
    f.done = false;
    f.tid = ref_uint3{i % block.x, (i / block.x) % block.y, i / (block.x * block.y)};
    if (f.stack.size() < kStack) f.stack.resize(kStack);
    getcontext(&f.ctx);
    f.ctx.uc_stack.ss_sp = f.stack.data();
    f.ctx.uc_stack.ss_size = f.stack.size();
    f.ctx.uc_link = &g_sched;
    makecontext(&f.ctx, trampoline, 0);
  }
  bool live = true;
  while (live) {
    live = false;
    for (unsigned i = 0; i < n; ++i) {
      if (g_fibers[i].done) continue;
      g_cur = (int)i;
      threadIdx = g_fibers[i].tid;
      swapcontext(&g_sched, &g_fibers[i].ctx);
      if (!g_fibers[i].done) live = true;
    }
  }
  g_cur = -1;
}

}  // namespace

void __syncthreads() {
  if (g_cur < 0) return;
  const int me = g_cur;
  swapcontext(&g_fibers[me].ctx, &g_sched);
  threadIdx = g_fibers[me].tid;  // restored by the scheduler too; kept for clarity
}

void* ref_simt_dynamic_smem() { return g_dyn.data(); }

namespace ref_simt {

void launch(ref_uint3 grid, ref_uint3 block, size_t dyn_smem_bytes, const std::function<void()>& body) {
  g_dyn.assign(std::max<size_t>(dyn_smem_bytes, 16), 0);
  g_body = &body;
  gridDim = grid;
  blockDim = block;
  for (unsigned z = 0; z < grid.z; ++z)
    for (unsigned y = 0; y < grid.y; ++y)
      for (unsigned x = 0; x < grid.x; ++x) {
        blockIdx = ref_uint3{x, y, z};
        run_block(block);
      }
  g_body = nullptr;
}

}  // namespace ref_simt

// ---- the reference's kernel text (generated, see header comment) ------------
namespace ref_spectrum {
#include "gen_spectrum.inc"
}
namespace ref_allmax {
#include "gen_allmax.inc"
}
namespace ref_fftproc {
#include "gen_fftproc.inc"
}

using ref_simt::dim;
using ref_simt::launch;

namespace {

// AllMaximaPipelineROCm::ExecutePrefixSum (all_maxima_pipeline_rocm.cpp:122-230),
// restated for host buffers: block_scan, recursion over block sums, block_add.
constexpr unsigned kScanLocal = 256, kScanBlock = 512;

void prefix_sum(const unsigned* input, unsigned* output, unsigned n_per_beam, unsigned beams) {
  const unsigned bpb = (n_per_beam + kScanBlock - 1) / kScanBlock;
  const unsigned total = beams * bpb;
  const size_t shm = (kScanBlock + 1) * sizeof(unsigned);
  if (bpb == 1) {
    launch(dim(total), dim(kScanLocal), shm, [&] {
      ref_allmax::block_scan(input, output, nullptr, n_per_beam, beams, bpb);
    });
    return;
  }
  std::vector<unsigned> sums(total), sums_scanned(total);
  unsigned* ps = sums.data();
  launch(dim(total), dim(kScanLocal), shm, [&] {
    ref_allmax::block_scan(input, output, ps, n_per_beam, beams, bpb);
  });
  prefix_sum(sums.data(), sums_scanned.data(), bpb, beams);
  const unsigned* pss = sums_scanned.data();
  launch(dim((n_per_beam + 255) / 256, beams), dim(256), 0, [&] {
    ref_allmax::block_add(output, pss, n_per_beam, beams, bpb, kScanBlock);
  });
}

}  // namespace

extern "C" {

// post_kernel_one_peak / post_kernel_two_peaks: grid = beams, block = 256
// (spectrum_post_op.hpp:93-98).  fft: interleaved float pairs [beams*nfft*2].
int ref_post_peaks(const float* fft, void* out, unsigned beams, unsigned nfft,
                   unsigned search_range, float fs, int two) {
  auto* f = reinterpret_cast<const ref_spectrum::float2_t*>(fft);
  auto* o = reinterpret_cast<ref_spectrum::MaxValue_t*>(out);
  launch(dim(beams), dim(256), 0, [&] {
    if (two)
      ref_spectrum::post_kernel_two_peaks(f, o, beams, nfft, search_range, fs);
    else
      ref_spectrum::post_kernel_one_peak(f, o, beams, nfft, search_range, fs);
  });
  return 0;
}

// compute_magnitudes over `total` elements (the relaunch with the correct
// grid, spectrum_processor_rocm.cpp:726-745).
int ref_compute_magnitudes(const float* fft, float* mags, unsigned total) {
  auto* f = reinterpret_cast<const ref_spectrum::float2_t*>(fft);
  launch(dim((total + 255) / 256), dim(256), 0, [&] { ref_spectrum::compute_magnitudes(f, mags, total); });
  return 0;
}

// AllMaximaPipelineROCm::Execute (all_maxima_pipeline_rocm.cpp:258-398):
// defaults, capacity, detect -> scan -> compact.  out: [beams * cap] MaxValue
// (entries beyond a beam's count are left as they were), counts: [beams]
// untruncated.  Returns the capacity used.
unsigned ref_all_maxima(const float* mags, const float* fft, unsigned beams, unsigned nfft,
                        float fs, unsigned start, unsigned end, unsigned max_per_beam,
                        void* out, unsigned* counts) {
  if (start == 0) start = 1;
  if (end == 0) end = nfft / 2;
  if (end >= nfft) end = nfft - 1;
  const size_t total = (size_t)beams * nfft;
  std::vector<unsigned> flags(total), scan(total);
  const unsigned cap = std::min((end - start) / 2, max_per_beam);
  unsigned* pf = flags.data();
  launch(dim((nfft + 255) / 256, beams), dim(256), 0, [&] {
    ref_allmax::detect_all_maxima(mags, pf, beams, nfft, start, end);
  });
  prefix_sum(flags.data(), scan.data(), nfft, beams);
  auto* f = reinterpret_cast<const ref_allmax::float2_t*>(fft);
  auto* o = reinterpret_cast<ref_allmax::MaxValue_t*>(out);
  const unsigned* ps = scan.data();
  launch(dim((nfft + 255) / 256, beams), dim(256), 0, [&] {
    ref_allmax::compact_maxima(f, mags, pf, ps, o, counts, beams, nfft, fs, cap, 0u);
  });
  return cap;
}

// complex_to_magnitude(_squared) and complex_to_mag_phase (1D, 256/block).
int ref_complex_to_magnitude(const float* in, float* out, float inv_n, unsigned total, int squared) {
  auto* z = reinterpret_cast<const ref_fftproc::float2_t*>(in);
  launch(dim((total + 255) / 256), dim(256), 0, [&] {
    if (squared)
      ref_fftproc::complex_to_magnitude_squared(z, out, inv_n, total);
    else
      ref_fftproc::complex_to_magnitude(z, out, inv_n, total);
  });
  return 0;
}

int ref_complex_to_mag_phase(const float* in, float* out, unsigned total) {
  auto* z = reinterpret_cast<const ref_fftproc::float2_t*>(in);
  auto* o = reinterpret_cast<ref_fftproc::float2_t*>(out);
  launch(dim((total + 255) / 256), dim(256), 0, [&] { ref_fftproc::complex_to_mag_phase(z, o, total); });
  return 0;
}

// memset + pad_data_windowed (PadDataOp::Execute, pad_data_op.hpp:86-131).
int ref_pad_windowed(const float* in, float* out, unsigned beams, unsigned n_point, unsigned nfft,
                     int window) {
  std::memset(out, 0, sizeof(float) * 2 * (size_t)beams * nfft);
  auto* x = reinterpret_cast<const ref_fftproc::float2_t*>(in);
  auto* y = reinterpret_cast<ref_fftproc::float2_t*>(out);
  launch(dim((n_point + 255) / 256, beams), dim(256), 0, [&] {
    if (window == 0)
      ref_fftproc::pad_data(x, y, n_point, nfft);
    else
      ref_fftproc::pad_data_windowed(x, y, n_point, nfft, window);
  });
  return 0;
}

}  // extern "C"
