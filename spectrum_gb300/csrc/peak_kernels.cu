// peak_kernels.cu — |X| / phase and the spectral peak search on a spectrum
// that is already in device memory.
//
//   magnitude_kernel      complex_to_magnitude(_squared) (fft_processor_kernels_rocm.hpp:142-174)
//   mag_phase_kernel      complex_to_mag_phase            (fft_processor_kernels_rocm.hpp:122-136)
//   one_two_peaks_kernel  post_kernel_one_peak / two_peaks (fft_kernel_sources_rocm.hpp:122-519)
//   all_maxima_kernel     detect_all_maxima + block_scan/block_add + compact_maxima
//                         (all_maxima_kernel_sources_rocm.hpp:57-264) as ONE single-pass
//                         kernel: the scan across tiles is a decoupled look-back.
//   topk_kernel           top-K strict local maxima (no reference counterpart)
//   noise_hist/select     per-beam noise threshold (no reference counterpart)
#include <cuda/atomic>

#include <cmath>

#include "spx_device.cuh"
#include "spx_internal.h"

namespace spx {

// ---------------------------------------------------------------------------
// |X| and {|X|, phase}
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256)
magnitude_kernel(const float2* __restrict__ in, float* __restrict__ out, uint64_t count,
                 float inv_n, int squared) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  const uint64_t i0 = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool vec = ((reinterpret_cast<uintptr_t>(in) & 15u) == 0) &&
                   ((reinterpret_cast<uintptr_t>(out) & 7u) == 0);
  if (vec) {
    const uint64_t npairs = count >> 1;
    const float4* in4 = reinterpret_cast<const float4*>(in);
    float2* out2 = reinterpret_cast<float2*>(out);
    for (uint64_t p = i0; p < npairs; p += stride) {
      const float4 v = __ldcs(in4 + p);
      float a = mag2_rn(make_float2(v.x, v.y));
      float b = mag2_rn(make_float2(v.z, v.w));
      if (!squared) {
        a = __fsqrt_rn(a);
        b = __fsqrt_rn(b);
      }
      __stcs(out2 + p, make_float2(__fmul_rn(a, inv_n), __fmul_rn(b, inv_n)));
    }
    if (i0 == 0 && (count & 1)) {
      const uint64_t t = count - 1;
      float a = mag2_rn(in[t]);
      if (!squared) a = __fsqrt_rn(a);
      out[t] = __fmul_rn(a, inv_n);
    }
  } else {
    for (uint64_t t = i0; t < count; t += stride) {
      float a = mag2_rn(in[t]);
      if (!squared) a = __fsqrt_rn(a);
      out[t] = __fmul_rn(a, inv_n);
    }
  }
}

__global__ void __launch_bounds__(256)
mag_phase_kernel(const float2* __restrict__ in, float2* __restrict__ out, uint64_t count) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < count; t += stride) {
    const float2 z = __ldcs(in + t);
    __stcs(out + t, make_float2(mag_rn(z), atan2f(z.y, z.x)));
  }
}

static unsigned grid_for(spx_ctx* ctx, uint64_t work, unsigned threads) {
  uint64_t blocks = (work + threads - 1) / threads;
  const uint64_t cap = (uint64_t)ctx->sm_count * 8;
  if (blocks > cap) blocks = cap;
  if (blocks == 0) blocks = 1;
  return (unsigned)blocks;
}

spx_status launch_magnitude(spx_ctx* ctx, const float2* d_in, float* d_out, uint64_t count,
                            float inv_n, int squared) {
  if (count == 0) return SPX_OK;
  magnitude_kernel<<<grid_for(ctx, (count + 1) / 2, 256), 256, 0, ctx->stream>>>(
      d_in, d_out, count, inv_n, squared);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? SPX_OK : cuda_fail(ctx, e, "launch magnitude_kernel");
}

spx_status launch_mag_phase(spx_ctx* ctx, const float2* d_in, float2* d_out, uint64_t count) {
  if (count == 0) return SPX_OK;
  mag_phase_kernel<<<grid_for(ctx, count, 256), 256, 0, ctx->stream>>>(d_in, d_out, count);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? SPX_OK : cuda_fail(ctx, e, "launch mag_phase_kernel");
}

// ---------------------------------------------------------------------------
// Shared peak helpers
// ---------------------------------------------------------------------------
SPX_DEV float phase_deg(float2 z) { return __fmul_rn(atan2f(z.y, z.x), kRadToDeg); }

// 3-point parabolic offset on magnitudes, clamped to [-0.5, 0.5], 0 when the
// curvature is below 1e-10 (fft_kernel_sources_rocm.hpp:229-239).
SPX_DEV bool parabolic(float yl, float yc, float yr, float* fo) {
  const float denom = __fadd_rn(__fsub_rn(yl, __fmul_rn(2.0f, yc)), yr);
  if (fabsf(denom) > 1e-10f) {
    float f = __fdiv_rn(__fmul_rn(0.5f, __fsub_rn(yl, yr)), denom);
    if (f < -0.5f) f = -0.5f;
    if (f > 0.5f) f = 0.5f;
    *fo = f;
    return true;
  }
  *fo = 0.0f;
  return false;
}

SPX_DEV uint64_t lane_max_u64(uint64_t v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const uint64_t w = __shfl_xor_sync(0xffffffffu, v, o);
    v = w > v ? w : v;
  }
  return v;
}

// ---------------------------------------------------------------------------
// ONE_PEAK / TWO_PEAKS
// ---------------------------------------------------------------------------
// Argmax key reproducing the reference's reduction order: a range is scanned
// by 256 threads, thread `lid` visiting offsets lid, lid+256, ... and keeping
// its first strict maximum; the shared-memory tree then merges local[lid]
// with local[lid + stride] for stride = 128 ... 1, keeping local[lid] on ties
// (fft_kernel_sources_rocm.hpp:151-192).  The last merge prefers even lids,
// the one before lid bit 1 = 0, and so on, so among equal magnitudes the
// winner has the smallest 8-bit-reversed lid, then the smallest offset.
// The key orders exactly that way under an unsigned max; NaN never wins (0).
SPX_DEV uint64_t one_two_key(float mag, uint32_t t) {
  if (!(mag >= 0.0f)) return 0ull;
  const uint32_t rev = __brev(t & 255u) & 0xFF000000u;  // bit-reversed lid in the top byte
  const uint32_t low = ~(rev | ((t >> 8) & 0xFFFFFFu));
  return ((uint64_t)__float_as_uint(mag) << 32) | low;
}
SPX_DEV uint32_t one_two_offset(uint64_t key) {
  const uint32_t low = ~(uint32_t)key;
  const uint32_t lid = __brev(low & 0xFF000000u);  // undo the reversal
  return ((low & 0xFFFFFFu) << 8) | lid;
}

// Writes the 4 MaxValue of one peak (interpolated, left, center, right)
// exactly as post_kernel_one_peak does (fft_kernel_sources_rocm.hpp:212-286).
SPX_DEV void write_peak4(const float2* __restrict__ f, uint32_t nfft, uint32_t ci, float fs,
                         bool mirror, MaxValueDev* o) {
  const float bw = __fdiv_rn(fs, (float)nfft);
  const float2 cv = f[ci];
  const float yc = mag_rn(cv);
  float2 lv = make_float2(0.f, 0.f), rv = make_float2(0.f, 0.f);
  float yl = 0.f, yr = 0.f;
  const bool hl = ci > 0, hr = ci < nfft - 1;
  if (hl) { lv = f[ci - 1]; yl = mag_rn(lv); }
  if (hr) { rv = f[ci + 1]; yr = mag_rn(rv); }
  float fo = 0.f;
  float rf = __fmul_rn((float)ci, bw);
  if (hl && hr) {
    if (parabolic(yl, yc, yr, &fo)) rf = __fmul_rn(__fadd_rn((float)ci, fo), bw);
  }
  if (mirror) rf = __fsub_rn(fs, rf);
  const float pc = phase_deg(cv);
  o[0] = MaxValueDev{ci, cv.x, cv.y, yc, pc, fo, rf, 0u};
  float rfl = hl ? __fmul_rn((float)(ci - 1), bw) : 0.f;
  if (mirror && hl) rfl = __fsub_rn(fs, rfl);
  o[1] = MaxValueDev{hl ? ci - 1 : 0u, lv.x, lv.y, yl, hl ? phase_deg(lv) : 0.f, 0.f, rfl, 0u};
  float rfc = __fmul_rn((float)ci, bw);
  if (mirror) rfc = __fsub_rn(fs, rfc);
  o[2] = MaxValueDev{ci, cv.x, cv.y, yc, pc, 0.f, rfc, 0u};
  float rfr = hr ? __fmul_rn((float)(ci + 1), bw) : 0.f;
  if (mirror && hr) rfr = __fsub_rn(fs, rfr);
  o[3] = MaxValueDev{hr ? ci + 1 : 0u, rv.x, rv.y, yr, hr ? phase_deg(rv) : 0.f, 0.f, rfr, 0u};
}

__global__ void __launch_bounds__(256)
one_two_peaks_kernel(const float2* __restrict__ fft, uint32_t nfft, uint32_t half, float fs,
                     int two_peaks, MaxValueDev* __restrict__ out) {
  __shared__ uint64_t sl[8], sr[8];
  const uint32_t beam = blockIdx.x;
  const float2* f = fft + (size_t)beam * nfft;
  const uint32_t r0 = nfft - half;
  uint64_t kl = 0, kr = 0;
  for (uint32_t t = threadIdx.x; t < half; t += blockDim.x) {
    const uint64_t a = one_two_key(mag_rn(f[t]), t);
    const uint64_t b = one_two_key(mag_rn(f[r0 + t]), t);
    kl = a > kl ? a : kl;
    kr = b > kr ? b : kr;
  }
  kl = lane_max_u64(kl);
  kr = lane_max_u64(kr);
  const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) { sl[warp] = kl; sr[warp] = kr; }
  __syncthreads();
  if (threadIdx.x != 0) return;
  for (uint32_t w = 1; w < (blockDim.x >> 5); ++w) {
    kl = sl[w] > kl ? sl[w] : kl;
    kr = sr[w] > kr ? sr[w] : kr;
  }
  kl = sl[0] > kl ? sl[0] : kl;
  kr = sr[0] > kr ? sr[0] : kr;
  // Decode; an empty (or all-NaN) range keeps the reference's initial values.
  const uint32_t il = kl ? one_two_offset(kl) : 0u;
  const float ml = kl ? __uint_as_float((uint32_t)(kl >> 32)) : -1.0f;
  const uint32_t ir = kr ? r0 + one_two_offset(kr) : r0;
  const float mr = kr ? __uint_as_float((uint32_t)(kr >> 32)) : -1.0f;
  if (two_peaks) {
    MaxValueDev* o = out + (size_t)beam * 8;
    write_peak4(f, nfft, il, fs, false, o);
    write_peak4(f, nfft, ir, fs, true, o + 4);
  } else {
    MaxValueDev* o = out + (size_t)beam * 4;
    const bool right = mr > ml;
    write_peak4(f, nfft, right ? ir : il, fs, right, o);
  }
}

spx_status launch_one_two(spx_ctx* ctx, const float2* d_fft, uint32_t beams, uint32_t nfft,
                          uint32_t search_range, float fs, int two_peaks, spx_max_value* d_out) {
  if (beams == 0) return SPX_OK;
  one_two_peaks_kernel<<<beams, 256, 0, ctx->stream>>>(d_fft, nfft, search_range / 2, fs,
                                                       two_peaks,
                                                       reinterpret_cast<MaxValueDev*>(d_out));
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? SPX_OK : cuda_fail(ctx, e, "launch one_two_peaks_kernel");
}

// ---------------------------------------------------------------------------
// All local maxima: detect + decoupled look-back scan + compact, one pass.
// ---------------------------------------------------------------------------
constexpr uint32_t kAmThreads = 256;
constexpr uint32_t kAmRounds = 8;
constexpr uint32_t kAmTile = kAmThreads * kAmRounds;  // bins per tile

// Tile status word: epoch (32) | flag (2) | count (30).  flag 1 = tile
// aggregate published, 2 = inclusive prefix published.  Words from another
// launch (other epoch) read as "not yet published", so no clearing is needed.
SPX_DEV uint64_t st_pack(uint32_t epoch, uint32_t flag, uint32_t v) {
  return ((uint64_t)epoch << 32) | ((uint64_t)flag << 30) | (v & 0x3FFFFFFFu);
}

struct AmArgs {
  const float* mag;    // may be null: |X| computed from fft
  const float2* fft;
  const float* thr;    // may be null
  MaxValueDev* out;
  uint32_t* counts;
  unsigned long long* status;
  uint32_t* ticket;
  uint32_t* err;
  uint32_t nfft, start, end, cap, tiles_per_beam, epoch, refine;
  float fs;
};

// Scan the tile: returns this tile's exclusive prefix within the beam.
// Thread 0 publishes the aggregate, then walks back over earlier tiles.
SPX_DEV uint32_t lookback(const AmArgs& a, uint32_t beam, uint32_t t, uint32_t agg) {
  using ref_t = cuda::atomic_ref<unsigned long long, cuda::thread_scope_device>;
  unsigned long long* st = a.status + (size_t)beam * a.tiles_per_beam;
  if (t == 0) {
    ref_t(st[0]).store(st_pack(a.epoch, 2, agg), cuda::memory_order_release);
    return 0;
  }
  ref_t(st[t]).store(st_pack(a.epoch, 1, agg), cuda::memory_order_release);
  uint32_t excl = 0;
  int p = (int)t - 1;
  const uint64_t t0 = globaltimer_ns();
  while (p >= 0) {
    const uint64_t v = ref_t(st[p]).load(cuda::memory_order_acquire);
    const uint32_t flag = (uint32_t)(v >> 30) & 3u;
    if ((uint32_t)(v >> 32) != a.epoch || flag == 0) {
      if (globaltimer_ns() - t0 > kSpinLimitNs) {
        atomicOr(a.err, kErrLookbackTimeout);
        break;
      }
      __nanosleep(32);
      continue;
    }
    excl += (uint32_t)v & 0x3FFFFFFFu;
    if (flag == 2) break;
    --p;
  }
  ref_t(st[t]).store(st_pack(a.epoch, 2, excl + agg), cuda::memory_order_release);
  return excl;
}

SPX_DEV MaxValueDev make_max(uint32_t bin, float2 z, float yl, float yc, float yr, float bw,
                             uint32_t refine) {
  float fo = 0.f;
  float rf = __fmul_rn((float)bin, bw);
  if (refine == SPX_REFINE_PARABOLIC) {
    if (parabolic(yl, yc, yr, &fo)) rf = __fmul_rn(__fadd_rn((float)bin, fo), bw);
  }
  return MaxValueDev{bin, z.x, z.y, yc, phase_deg(z), fo, rf, 0u};
}

__global__ void __launch_bounds__(kAmThreads)
all_maxima_kernel(AmArgs a) {
  __shared__ float smag[kAmTile + 2];
  __shared__ uint32_t sball[kAmRounds][kAmThreads / 32];
  __shared__ uint32_t spre[kAmRounds][kAmThreads / 32];
  __shared__ uint32_t s_tile, s_agg, s_excl;
  const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) s_tile = atomicAdd(a.ticket, 1u);
  __syncthreads();
  const uint32_t tile = s_tile;
  const uint32_t beam = tile / a.tiles_per_beam, t = tile - beam * a.tiles_per_beam;
  const uint32_t lo = a.start + t * kAmTile;
  const uint32_t hi = min(lo + kAmTile, a.end);
  const size_t bb = (size_t)beam * a.nfft;
  const uint32_t nload = hi > lo ? hi - lo + 2 : 0;  // bins [lo-1, hi+1)
  for (uint32_t i = tid; i < nload; i += kAmThreads) {
    const uint32_t bin = lo - 1 + i;
    smag[i] = a.mag ? __ldg(a.mag + bb + bin) : mag_rn(__ldg(a.fft + bb + bin));
  }
  __syncthreads();
  const float thr = a.thr ? a.thr[beam] : -INFINITY;
  // Round u covers bins lo + u*256 + tid: consecutive threads, consecutive bins.
  uint32_t bits = 0;
#pragma unroll
  for (uint32_t u = 0; u < kAmRounds; ++u) {
    const uint32_t i = u * kAmThreads + tid;
    bool f = false;
    if (lo + i < hi) {
      const float c = smag[i + 1];
      f = (c > smag[i]) && (c > smag[i + 2]) && (c > thr);
    }
    const uint32_t b = __ballot_sync(0xffffffffu, f);
    if (f) bits |= 1u << u;
    if (lane == 0) sball[u][warp] = b;
  }
  __syncthreads();
  // Exclusive prefix over (round, warp) in bin order; warp 0 scans 64 counts.
  if (warp == 0) {
    uint32_t c0 = __popc(sball[lane >> 3][lane & 7]);
    uint32_t c1 = __popc(sball[4 + (lane >> 3)][lane & 7]);
    uint32_t x0 = c0, x1 = c1;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y0 = __shfl_up_sync(0xffffffffu, x0, o);
      const uint32_t y1 = __shfl_up_sync(0xffffffffu, x1, o);
      if (lane >= (uint32_t)o) { x0 += y0; x1 += y1; }
    }
    const uint32_t tot0 = __shfl_sync(0xffffffffu, x0, 31);
    spre[lane >> 3][lane & 7] = x0 - c0;
    spre[4 + (lane >> 3)][lane & 7] = tot0 + x1 - c1;
    const uint32_t agg = tot0 + __shfl_sync(0xffffffffu, x1, 31);
    if (lane == 0) {
      s_agg = agg;
      s_excl = lookback(a, beam, t, agg);
    }
  }
  __syncthreads();
  const uint32_t excl = s_excl;
  if (t == a.tiles_per_beam - 1 && tid == 0) a.counts[beam] = excl + s_agg;
  if (bits) {
    const float bw = __fdiv_rn(a.fs, (float)a.nfft);
    const uint32_t lt = (1u << lane) - 1u;
    MaxValueDev* o = a.out + (size_t)beam * a.cap;
#pragma unroll
    for (uint32_t u = 0; u < kAmRounds; ++u) {
      if (bits & (1u << u)) {
        const uint32_t rank = excl + spre[u][warp] + __popc(sball[u][warp] & lt);
        if (rank < a.cap) {
          const uint32_t i = u * kAmThreads + tid;
          const uint32_t bin = lo + i;
          o[rank] = make_max(bin, __ldg(a.fft + bb + bin), smag[i], smag[i + 1], smag[i + 2],
                             bw, a.refine);
        }
      }
    }
  }
}

// Real samples -> complex samples with zero imaginary part (input of the
// real-input transform).
__global__ void widen_real_kernel(const float* __restrict__ in, float2* __restrict__ out, uint64_t n) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
    out[i] = make_float2(__ldg(in + i), 0.0f);
}

spx_status launch_widen_real(spx_ctx* ctx, const float* d_in, float2* d_out, uint64_t n) {
  const unsigned grid = (unsigned)std::min<uint64_t>((n + 255) / 256, (uint64_t)ctx->sm_count * 16);
  widen_real_kernel<<<grid, 256, 0, ctx->stream>>>(d_in, d_out, n);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? SPX_OK : cuda_fail(ctx, e, "launch widen_real_kernel");
}

// Self-test of the bounded wait: one thread waits, as tile 1 of a beam, on
// tile 0's status word, which holds another epoch and is never published, so
// the wait ends at its time bound and sets kErrLookbackTimeout.
__global__ void lookback_timeout_probe_kernel(unsigned long long* status, uint32_t* err, uint32_t epoch) {
  AmArgs a{};
  a.status = status;
  a.err = err;
  a.tiles_per_beam = 2;
  a.epoch = epoch;
  lookback(a, 0, 1, 0);
}

spx_status launch_lookback_timeout_probe(spx_ctx* ctx, unsigned long long* d_status) {
  cudaError_t e = cudaMemsetAsync(d_status, 0, 2 * sizeof(unsigned long long), ctx->stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "lookback probe memset");
  lookback_timeout_probe_kernel<<<1, 1, 0, ctx->stream>>>(d_status, ctx->d_error, 1u);
  e = cudaGetLastError();
  return e == cudaSuccess ? SPX_OK : cuda_fail(ctx, e, "launch lookback_timeout_probe_kernel");
}

spx_status launch_all_maxima(spx_ctx* ctx, const float* d_mag, const float2* d_fft,
                             uint32_t beams, uint32_t nfft, uint32_t start, uint32_t end,
                             uint32_t cap, float fs, uint32_t refine, const float* d_thr,
                             spx_max_value* d_out, uint32_t* d_counts) {
  if (beams == 0) return SPX_OK;
  const uint32_t span = end > start ? end - start : 0;
  uint32_t tpb = (span + kAmTile - 1) / kAmTile;
  if (tpb == 0) tpb = 1;
  const uint64_t tiles = (uint64_t)tpb * beams;
  if (tiles > 0x7FFFFFFFull) return fail(ctx, SPX_ERR_INVALID_ARG, "all_maxima: too many tiles");
  const size_t status_bytes = ((size_t)tiles * 8 + 255) & ~(size_t)255;
  void* scratch = nullptr;
  spx_status st = get_scratch(ctx, kSlotWork, status_bytes + 256, &scratch);
  if (st != SPX_OK) return st;
  AmArgs a{};
  a.mag = d_mag;
  a.fft = d_fft;
  a.thr = d_thr;
  a.out = reinterpret_cast<MaxValueDev*>(d_out);
  a.counts = d_counts;
  a.status = reinterpret_cast<unsigned long long*>(scratch);
  a.ticket = reinterpret_cast<uint32_t*>(static_cast<char*>(scratch) + status_bytes);
  a.err = ctx->d_error;
  a.nfft = nfft;
  a.start = start;
  a.end = end;
  a.cap = cap;
  a.tiles_per_beam = tpb;
  a.epoch = ++ctx->epoch;
  if (a.epoch == 0) a.epoch = ++ctx->epoch;  // 0 is never a valid epoch
  a.refine = refine;
  a.fs = fs;
  // Status words and the ticket counter start at zero on every launch (a
  // freshly allocated scratch buffer may hold any bits).
  cudaError_t e = cudaMemsetAsync(scratch, 0, status_bytes + sizeof(uint32_t), ctx->stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaMemsetAsync(look-back status)");
  all_maxima_kernel<<<(unsigned)tiles, kAmThreads, 0, ctx->stream>>>(a);
  e = cudaGetLastError();
  return e == cudaSuccess ? SPX_OK : cuda_fail(ctx, e, "launch all_maxima_kernel");
}

// Same launch with caller-provided scratch (status words of `tiles` tiles,
// then one 32-bit ticket); allocates nothing.  Used by the allocation-free
// entry point (spx_noalloc.cu).
spx_status launch_all_maxima_in(spx_ctx* ctx, const float* d_mag, const float2* d_fft,
                                uint32_t beams, uint32_t nfft, uint32_t start, uint32_t end,
                                uint32_t cap, float fs, uint32_t refine, spx_max_value* d_out,
                                uint32_t* d_counts, void* scratch, size_t scratch_bytes) {
  if (beams == 0) return SPX_OK;
  const uint64_t tiles = all_maxima_tiles(beams, start, end);
  const size_t status_bytes = ((size_t)tiles * 8 + 255) & ~(size_t)255;
  if (status_bytes + sizeof(uint32_t) > scratch_bytes)
    return fail(ctx, SPX_ERR_INVALID_ARG, "all_maxima: scratch too small");
  AmArgs a{};
  a.mag = d_mag;
  a.fft = d_fft;
  a.thr = nullptr;
  a.out = reinterpret_cast<MaxValueDev*>(d_out);
  a.counts = d_counts;
  a.status = reinterpret_cast<unsigned long long*>(scratch);
  a.ticket = reinterpret_cast<uint32_t*>(static_cast<char*>(scratch) + status_bytes);
  a.err = ctx->d_error;
  a.nfft = nfft;
  a.start = start;
  a.end = end;
  a.cap = cap;
  a.tiles_per_beam = (uint32_t)(tiles / beams);
  a.epoch = 1;
  a.refine = refine;
  a.fs = fs;
  cudaError_t e = cudaMemsetAsync(scratch, 0, status_bytes + sizeof(uint32_t), ctx->stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaMemsetAsync(look-back status)");
  all_maxima_kernel<<<(unsigned)tiles, kAmThreads, 0, ctx->stream>>>(a);
  e = cudaGetLastError();
  return e == cudaSuccess ? SPX_OK : cuda_fail(ctx, e, "launch all_maxima_kernel");
}

uint64_t all_maxima_tiles(uint32_t beams, uint32_t start, uint32_t end) {
  const uint32_t span = end > start ? end - start : 0;
  uint64_t tpb = (span + kAmTile - 1) / kAmTile;
  if (tpb == 0) tpb = 1;
  return tpb * beams;
}

// ---------------------------------------------------------------------------
// Top-K strict local maxima, one CTA per beam, one sorted list per warp.
// ---------------------------------------------------------------------------
constexpr uint32_t kTkThreads = 256;
constexpr uint32_t kTkWarps = kTkThreads / 32;
constexpr uint32_t kTkRun = 8;  // runs of 32 bins per warp step

// Key orders by |X| descending, then bin ascending; 0 = empty slot.
SPX_DEV uint64_t topk_key(float mag, uint32_t bin) {
  return ((uint64_t)__float_as_uint(mag) << 32) | (uint32_t)(~bin);
}

SPX_DEV float mag_at(const float* mag, const float2* fft, size_t i) {
  return mag ? __ldg(mag + i) : mag_rn(__ldg(fft + i));
}

__global__ void __launch_bounds__(kTkThreads)
topk_kernel(const float* __restrict__ mag, const float2* __restrict__ fft, uint32_t nfft,
            uint32_t start, uint32_t end, uint32_t K, float fs, uint32_t refine,
            const float* __restrict__ thrs, MaxValueDev* __restrict__ out,
            uint32_t* __restrict__ counts) {
  __shared__ uint64_t lists[kTkWarps][32];
  const uint32_t beam = blockIdx.x;
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const size_t bb = (size_t)beam * nfft;
  const float thr = thrs ? thrs[beam] : -INFINITY;
  uint64_t mine = 0;  // this lane's list entry
  // A warp step covers kTkRun runs of 32 consecutive bins (bin base + 32j +
  // lane): kTkRun loads in flight per lane, 128- or 256-byte warp reads, each
  // |X| computed once and the neighbours taken from the adjacent lanes (or
  // runs; two loads at the step's edges).  Bins start - 1 .. end are read.
  for (uint32_t base = start + warp * 32 * kTkRun; base < end; base += kTkThreads * kTkRun) {
    float m[kTkRun];
    if (mag) {
#pragma unroll
      for (uint32_t j = 0; j < kTkRun; ++j) {
        const uint32_t b = base + 32 * j + lane;
        m[j] = b <= end ? __ldg(mag + bb + b) : 0.f;
      }
    } else {
      float2 z[kTkRun];
#pragma unroll
      for (uint32_t j = 0; j < kTkRun; ++j) {
        const uint32_t b = base + 32 * j + lane;
        z[j] = b <= end ? __ldg(fft + bb + b) : make_float2(0.f, 0.f);
      }
#pragma unroll
      for (uint32_t j = 0; j < kTkRun; ++j) m[j] = mag_rn(z[j]);
    }
    float edge = 0.f;  // lane 0: bin base - 1; lane 31: bin base + 32 kTkRun
    if (lane == 0) edge = mag_at(mag, fft, bb + base - 1);
    if (lane == 31 && base + 32 * kTkRun <= end) edge = mag_at(mag, fft, bb + base + 32 * kTkRun);
#pragma unroll
    for (uint32_t j = 0; j < kTkRun; ++j) {
      const uint32_t b = base + 32 * j + lane;
      const float prev_last = __shfl_sync(0xffffffffu, m[j == 0 ? 0 : j - 1], 31);
      const float next_first = __shfl_sync(0xffffffffu, m[j + 1 < kTkRun ? j + 1 : j], 0);
      float l = __shfl_up_sync(0xffffffffu, m[j], 1), r = __shfl_down_sync(0xffffffffu, m[j], 1);
      if (lane == 0) l = j == 0 ? edge : prev_last;
      if (lane == 31) r = j + 1 == kTkRun ? edge : next_first;
      const float c = m[j];
      const bool cand = b < end && c > l && c > r && c > thr;
      const uint64_t key = topk_key(c, b);
      const uint64_t kth = __shfl_sync(0xffffffffu, mine, K - 1);
      uint32_t want = __ballot_sync(0xffffffffu, cand && key > kth);
      while (want) {
        const int src = __ffs(want) - 1;
        want &= want - 1;
        const uint64_t x = __shfl_sync(0xffffffffu, key, src);
        mine = warp_list_insert(mine, x, lane);
      }
    }
  }
  mine = merge_warp_lists(&lists[0][0], mine, kTkWarps, K, warp, lane);
  if (warp != 0) return;
  const uint32_t n = __popc(__ballot_sync(0xffffffffu, lane < K && mine != 0));
  if (lane == 0) counts[beam] = n;
  if (lane < n) {
    const uint32_t bin = ~(uint32_t)mine;
    const float bw = __fdiv_rn(fs, (float)nfft);
    const float yc = __uint_as_float((uint32_t)(mine >> 32));
    const float yl = mag_at(mag, fft, bb + bin - 1);
    const float yr = mag_at(mag, fft, bb + bin + 1);
    out[(size_t)beam * K + lane] = make_max(bin, __ldg(fft + bb + bin), yl, yc, yr, bw, refine);
  }
}

spx_status launch_topk(spx_ctx* ctx, const float* d_mag, const float2* d_fft, uint32_t beams,
                       uint32_t nfft, uint32_t start, uint32_t end, uint32_t k, float fs,
                       uint32_t refine, const float* d_thr, spx_max_value* d_out,
                       uint32_t* d_counts) {
  if (beams == 0) return SPX_OK;
  topk_kernel<<<beams, kTkThreads, 0, ctx->stream>>>(d_mag, d_fft, nfft, start, end, k, fs,
                                                     refine, d_thr,
                                                     reinterpret_cast<MaxValueDev*>(d_out),
                                                     d_counts);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? SPX_OK : cuda_fail(ctx, e, "launch topk_kernel");
}

// ---------------------------------------------------------------------------
// Noise threshold: histogram-interpolated median of |X| over [start, end).
//   bucket(m) = (bits(m) & 0x7fffffff) >> 19   (4096 buckets: exponent + 4 mantissa bits)
//   r = (n - 1) / 2; bucket b holds rank r; lo/hi = bucket edges;
//   frac = ((float)(r - below) + 0.5f) / (float)h[b];  med = lo + (hi - lo) * frac
//   thr = med * factor                      (all FP32, each step rounded)
// ---------------------------------------------------------------------------
constexpr uint32_t kHistBins = 4096;
constexpr uint32_t kHistTile = 8192;

SPX_DEV uint32_t noise_bucket(float m) { return (__float_as_uint(m) & 0x7fffffffu) >> 19; }

__global__ void __launch_bounds__(256)
noise_hist_kernel(const float* __restrict__ mag, const float2* __restrict__ fft, uint32_t nfft,
                  uint32_t start, uint32_t end, uint32_t tiles_per_beam,
                  uint32_t* __restrict__ hist) {
  __shared__ uint32_t h[kHistBins];
  for (uint32_t i = threadIdx.x; i < kHistBins; i += blockDim.x) h[i] = 0;
  __syncthreads();
  const uint32_t beam = blockIdx.x / tiles_per_beam, t = blockIdx.x % tiles_per_beam;
  const size_t bb = (size_t)beam * nfft;
  const uint32_t lo = start + t * kHistTile, hi = min(lo + kHistTile, end);
  for (uint32_t bin = lo + threadIdx.x; bin < hi; bin += blockDim.x)
    atomicAdd(&h[noise_bucket(mag_at(mag, fft, bb + bin))], 1u);
  __syncthreads();
  uint32_t* g = hist + (size_t)beam * kHistBins;
  for (uint32_t i = threadIdx.x; i < kHistBins; i += blockDim.x)
    if (h[i]) atomicAdd(&g[i], h[i]);
}

__global__ void __launch_bounds__(1024)
noise_select_kernel(const uint32_t* __restrict__ hist, uint32_t n, float factor,
                    float* __restrict__ thr) {
  __shared__ uint32_t wsum[32];
  __shared__ uint32_t s_bucket, s_below;
  const uint32_t beam = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) {
    s_bucket = 0xFFFFFFFFu;
    s_below = 0;
  }
  const uint32_t* h = hist + (size_t)beam * kHistBins;
  // 4 buckets per thread, block-wide exclusive scan in bucket order.
  uint32_t c[4], s = 0;
#pragma unroll
  for (int j = 0; j < 4; ++j) { c[j] = h[tid * 4 + j]; s += c[j]; }
  uint32_t x = s;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= (uint32_t)o) x += y;
  }
  if (lane == 31) wsum[warp] = x;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = wsum[lane], v = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, v, o);
      if (lane >= (uint32_t)o) v += y;
    }
    wsum[lane] = v - w;
  }
  __syncthreads();
  const uint32_t r = (n - 1) / 2;
  uint32_t below = wsum[warp] + x - s;
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    if (below <= r && r < below + c[j]) { s_bucket = tid * 4 + j; s_below = below; }
    below += c[j];
  }
  __syncthreads();
  if (tid == 0) {
    if (n == 0 || s_bucket == 0xFFFFFFFFu) {
      thr[beam] = INFINITY;
      return;
    }
    const uint32_t b = s_bucket;
    const float lo = __uint_as_float(b << 19);
    const float hi = __uint_as_float((b + 1) << 19);
    const float frac = __fdiv_rn(__fadd_rn((float)(r - s_below), 0.5f), (float)h[b]);
    const float med = __fadd_rn(lo, __fmul_rn(__fsub_rn(hi, lo), frac));
    thr[beam] = __fmul_rn(med, factor);
  }
}

spx_status launch_noise_threshold(spx_ctx* ctx, const float* d_mag, const float2* d_fft,
                                  uint32_t beams, uint32_t nfft, uint32_t start, uint32_t end,
                                  float factor, float* d_thr) {
  if (beams == 0) return SPX_OK;
  const uint32_t n = end > start ? end - start : 0;
  uint32_t tpb = (n + kHistTile - 1) / kHistTile;
  if (tpb == 0) tpb = 1;
  void* scratch = nullptr;
  const size_t hbytes = (size_t)beams * kHistBins * sizeof(uint32_t);
  spx_status st = get_scratch(ctx, kSlotWork, hbytes, &scratch);
  if (st != SPX_OK) return st;
  uint32_t* hist = static_cast<uint32_t*>(scratch);
  cudaError_t e = cudaMemsetAsync(hist, 0, hbytes, ctx->stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaMemsetAsync(hist)");
  noise_hist_kernel<<<tpb * beams, 256, 0, ctx->stream>>>(d_mag, d_fft, nfft, start, end, tpb,
                                                          hist);
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(ctx, e, "launch noise_hist_kernel");
  noise_select_kernel<<<beams, 1024, 0, ctx->stream>>>(hist, n, factor, d_thr);
  e = cudaGetLastError();
  return e == cudaSuccess ? SPX_OK : cuda_fail(ctx, e, "launch noise_select_kernel");
}

}  // namespace spx
