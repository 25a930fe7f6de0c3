// spx_geom.h — FFT geometry passed by value to the kernels.
#pragma once

#include <stdint.h>

namespace spx {

// Error word bits written by kernels into spx_ctx::d_error.
constexpr uint32_t kErrLookbackTimeout = 1u;  // a bounded device-side wait gave up (look-back, beam group barrier)

constexpr int kMaxPass = 12;
constexpr uint32_t kMaxLocal = 16384;   // points per CTA (one local FFT)
constexpr uint32_t kPrefLocalCluster = 16384;  // preferred points per CTA when C > 1 (measured fastest on GB300)
constexpr int kEPTDefault = 16;         // points held per thread per pass (16 or 32)
// Dynamic shared memory the FFT kernels may ask for: a padded 16384-point
// local FFT (17408 elements) plus the fused kernels' histogram and lists.
constexpr uint32_t kMaxFftSmem = (16384u + 1024u) * 8u + 32768u;

// nfft = C * M.  The M-point local FFT runs npass Stockham passes; pass p
// has radix radix[p], input stride ns[p] (product of earlier radices) and
// its twiddles at tw_local + twoff[p].
// Twiddle rows stored per Stockham pass of radix R: W^{rk}, r = 1..R-1,
// except radix 4, which stores W^k only and forms W^2k = (W^k)^2 and
// W^3k = W^2k W^k in the pass: the last pass of a 16384-point FFT reads a
// 32 KB table instead of 96 KB, which keeps it in L1 beside the window.
constexpr uint32_t tw_rows(uint32_t R) { return R == 4 ? 1u : R - 1u; }
// A radix-4 pass with Ns >= kTwSplitNs stores W^k = W_{4 Ns}^k (k < Ns) as
// two factors, lo[l] = W^l (l < 64) then hi[j] = W^{64 j} (j < ceil(Ns / 64)),
// and forms W^k = hi[k >> 6] * lo[k & 63] (tw4 in fft_core.cuh): the last
// pass of a 16384-point FFT reads 1 KB of table instead of 32 KB, so the
// other passes' twiddles and the window stay in L1.
constexpr uint32_t kTwSplitNs = 1024;
constexpr bool tw_split(uint32_t R, uint32_t Ns) { return R == 4 && Ns >= kTwSplitNs; }
// Table entries of a pass of radix R and stride Ns.
constexpr uint32_t tw_entries(uint32_t R, uint32_t Ns) {
  return tw_split(R, Ns) ? 64u + (Ns + 63u) / 64u : Ns * tw_rows(R);
}

struct FftGeom {
  uint32_t nfft;
  uint32_t C;       // CTAs per beam (cluster size)
  uint32_t M;       // local FFT length
  uint32_t Mpad;    // shared-memory elements of the local FFT, sw_len(M) (spx_device.cuh)
  uint32_t T;       // threads per CTA
  uint32_t ept;     // points per thread (kernel instantiation: 16 or 32)
  uint32_t npass;
  uint32_t radix[kMaxPass];
  uint32_t ns[kMaxPass];
  uint32_t twoff[kMaxPass];
  uint32_t nsmagic[kMaxPass];  // ceil(2^32 / ns[p]) (0 for ns = 1): j mod ns = j - ns * umulhi(j, magic)
  // Set per launch (0 in plans): beams in the launch and the L2 prefetch
  // distance in beams (the beams resident at once; 0 = no prefetch).
  uint32_t beams;
  uint32_t ahead;
};

}  // namespace spx
