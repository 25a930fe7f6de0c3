// spx_noalloc.cu — an all-maxima search that allocates nothing.
//
// Who needs it: callers that must not allocate device memory while they
// run.  Examples are a real-time receive loop that reserves all of its GPU
// memory at start-up and forbids cudaMalloc afterwards (an allocation can
// stall on a device-wide synchronisation), or a host framework that owns
// every byte of device memory through its own pool.  spx_all_maxima grows a
// context scratch buffer on demand with cudaMalloc, so it cannot serve them.
//
// How: the look-back status words and the tile ticket live in one
// file-scope __device__ array of kNoAllocScratchBytes (256 KiB + 256 B),
// which every GPU that loads this library holds until the process exits.
// Host code cannot use the array's name as a device address, so the first
// call on each device (with that device current) resolves it once with
// cudaGetSymbolAddress and caches the pointer; make that first call before
// any stream capture.  Each call clears the status words and ticket with
// cudaMemsetAsync on the context's stream.  All calls share the array:
// calls whose kernels overlap on the GPU (different streams, or another
// host thread) race and corrupt each other's results; order them on one
// stream.
#include <mutex>

#include "spx_internal.h"

namespace spx {
namespace {

constexpr uint32_t kNoAllocMaxTiles = 32768;  // 2048 search bins per tile
constexpr size_t kNoAllocScratchBytes = (size_t)kNoAllocMaxTiles * 8 + 256;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_addr[kMaxDevices] = {};

// Device address of g_noalloc_scratch on the current device (resolved once).
spx_status scratch_address(spx_ctx* ctx, void** out) {
  if (ctx->device < 0 || ctx->device >= kMaxDevices)
    return fail(ctx, SPX_ERR_NO_DEVICE, "spx_all_maxima_noalloc: device ordinal out of range");
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_addr[ctx->device]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) return cuda_fail(ctx, e, "cudaGetSymbolAddress(no-alloc scratch)");
    g_addr[ctx->device] = p;
  }
  *out = g_addr[ctx->device];
  return SPX_OK;
}

}  // namespace
}  // namespace spx

using namespace spx;

extern "C" spx_status spx_all_maxima_noalloc(spx_ctx* ctx, const float* d_mag, const void* d_fft,
                                             uint32_t beams, uint32_t nfft,
                                             const spx_peak_params* params,
                                             spx_max_value* d_out, uint32_t* d_counts) {
  if (!ctx) return SPX_ERR_INVALID_ARG;
  if (!params) return fail(ctx, SPX_ERR_INVALID_ARG, "params is null");
  if (nfft < 3) return fail(ctx, SPX_ERR_INVALID_ARG, "nfft must be >= 3 for a peak search");
  if (params->refine > SPX_REFINE_PARABOLIC)
    return fail(ctx, SPX_ERR_INVALID_ARG, "unknown refine mode");
  if (params->thresh_sigma != 0.0f)
    return fail(ctx, SPX_ERR_INVALID_ARG,
                "spx_all_maxima_noalloc: thresh_sigma must be 0 (the noise threshold needs "
                "per-beam histogram scratch; use spx_all_maxima)");
  if (beams == 0) return SPX_OK;
  if (!d_fft || !d_counts)
    return fail(ctx, SPX_ERR_INVALID_ARG, "spx_all_maxima_noalloc: fft_data and counts are required");
  uint32_t start = 0, end = 0, cap = 0;
  spx_all_maxima_capacity(nfft, params->search_start, params->search_end, params->max_per_beam,
                          &start, &end, &cap);
  if (cap > 0 && !d_out)
    return fail(ctx, SPX_ERR_INVALID_ARG, "spx_all_maxima_noalloc: out is null");
  const uint64_t tiles = all_maxima_tiles(beams, start, end);
  if (tiles > kNoAllocMaxTiles)
    return fail(ctx, SPX_ERR_INVALID_ARG,
                "spx_all_maxima_noalloc: beams * ceil((end - start) / 2048) = " +
                    std::to_string(tiles) + " exceeds the fixed scratch limit of " +
                    std::to_string(kNoAllocMaxTiles) + " tiles");
  int prev = -1;
  if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
  if (prev != ctx->device && cudaSetDevice(ctx->device) != cudaSuccess)
    return fail(ctx, SPX_ERR_NO_DEVICE, "cudaSetDevice failed");
  void* scratch = nullptr;
  spx_status st = scratch_address(ctx, &scratch);
  if (st == SPX_OK)
    st = launch_all_maxima_in(ctx, d_mag, static_cast<const float2*>(d_fft), beams, nfft, start,
                              end, cap, params->sample_rate, params->refine, d_out, d_counts,
                              scratch, kNoAllocScratchBytes);
  if (prev >= 0 && prev != ctx->device) cudaSetDevice(prev);
  return st;
}
