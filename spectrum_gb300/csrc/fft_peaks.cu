// fft_peaks.cu — fused window + zero pad + FFT + |X| + noise threshold +
// peak search: the spectrum of a beam never leaves the chip.
//
// Replaces, for one beam per CTA (nfft <= 16384) or per cluster of C CTAs:
//   PadDataOp + hipfftExecC2C + ComputeMagnitudesOp + AllMaximaPipelineROCm
//   (src/fft_func/src/spectrum_processor_rocm.cpp:444-543,
//    src/fft_func/src/all_maxima_pipeline_rocm.cpp:258-472)
// with the noise threshold and parabolic refinement of this build.
//
// Modes:
//   ALL  + threshold : every strict local maximum of |X| in [start, end) above
//                      the per-beam threshold, compacted in bin order.
//   TOPK (C == 1)    : the K largest strict local maxima (optionally above the
//                      threshold), |X| descending, ties by lower bin.
// Results are bit-identical to spx_fft (COMPLEX) followed by spx_all_maxima /
// spx_topk: the same FFT code, |X| = sqrt_rn(re*re + im*im), the same
// histogram-median threshold and the same comparisons.
//
// C > 1 (the beam's bins k = c + C*i are spread over the cluster): after the
// cluster barrier that completes the beam's noise histogram every spectrum is
// final, so each CTA tests its bins above the threshold (few) against both
// neighbours read from the neighbours' CTAs (distributed shared memory) and
// keeps their magnitudes for the refinement; maxima bitmaps go through
// device memory, and after one more barrier every CTA ranks its maxima by a
// prefix popcount over the beam's maxima bitmap in bin order.
#include <cuda/atomic>

#include "fft_core.cuh"
#include "spx_internal.h"

namespace spx {

constexpr uint32_t kHist = 4096;  // noise-histogram buckets (exponent + 4 mantissa bits)
constexpr uint32_t kList = 1024;  // hot bins classified per round (C > 1); >= threads per CTA

struct FusedArgs {
  const float2* in;
  const float* win;
  const float2* tw_local;
  const float2* tw_cross;
  float2* xch;              // exchange slots (C > 1), one per beam
  uint32_t* ghist;          // [beams][4096] per-beam histograms (C > 1), zeroed by the host
  uint32_t* gbits;          // [beams][nfft/32 + C] maxima bitmaps (C > 1)
  MaxValueDev* out;
  uint32_t* counts;
  uint32_t n_point, start, end, cap, mode, K, refine;
  float fs, factor;         // factor <= 0: no threshold
};

SPX_DEV uint32_t bucket_of(float m) { return (__float_as_uint(m) & 0x7fffffffu) >> 19; }

// Histogram-interpolated median * factor from a 4096-bucket histogram in
// shared memory (identical arithmetic to noise_select_kernel).  All threads
// of the CTA call it; returns the threshold to every thread.
SPX_DEV float threshold_from_hist(const uint32_t* h, uint32_t n, float factor, uint32_t* s_red) {
  const uint32_t tid = threadIdx.x, T = blockDim.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t per = kHist / T;  // T divides 4096 (T in 32..1024, power of two)
  uint32_t sum = 0;
  for (uint32_t j = 0; j < per; ++j) sum += h[tid * per + j];
  uint32_t x = sum;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= (uint32_t)o) x += y;
  }
  if (lane == 31) s_red[warp] = x;
  __syncthreads();
  if (warp == 0) {
    const uint32_t nw = T >> 5;
    uint32_t w = lane < nw ? s_red[lane] : 0u, v = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, v, o);
      if (lane >= (uint32_t)o) v += y;
    }
    if (lane < nw) s_red[32 + lane] = v - w;
    if (lane == 0) { s_red[64] = 0xFFFFFFFFu; s_red[65] = 0; }
  }
  __syncthreads();
  const uint32_t r = (n - 1) / 2;
  uint32_t below = s_red[32 + warp] + x - sum;
  for (uint32_t j = 0; j < per; ++j) {
    const uint32_t c = h[tid * per + j];
    if (below <= r && r < below + c) { s_red[64] = tid * per + j; s_red[65] = below; }
    below += c;
  }
  __syncthreads();
  const uint32_t b = s_red[64];
  float thr = INFINITY;
  if (n > 0 && b != 0xFFFFFFFFu) {
    const float lo = __uint_as_float(b << 19);
    const float hi = __uint_as_float((b + 1) << 19);
    const float frac = __fdiv_rn(__fadd_rn((float)(r - s_red[65]), 0.5f), (float)h[b]);
    const float med = __fadd_rn(lo, __fmul_rn(__fsub_rn(hi, lo), frac));
    thr = __fmul_rn(med, factor);
  }
  __syncthreads();  // s_red reused by the caller
  return thr;
}

SPX_DEV MaxValueDev fused_max(uint32_t bin, float2 z, float yl, float yc, float yr, float bw,
                              uint32_t refine) {
  float fo = 0.f;
  float rf = __fmul_rn((float)bin, bw);
  if (refine == SPX_REFINE_PARABOLIC) {
    const float denom = __fadd_rn(__fsub_rn(yl, __fmul_rn(2.0f, yc)), yr);
    if (fabsf(denom) > 1e-10f) {
      float f = __fdiv_rn(__fmul_rn(0.5f, __fsub_rn(yl, yr)), denom);
      if (f < -0.5f) f = -0.5f;
      if (f > 0.5f) f = 0.5f;
      fo = f;
      rf = __fmul_rn(__fadd_rn((float)bin, fo), bw);
    }
  }
  return MaxValueDev{bin, z.x, z.y, yc, __fmul_rn(atan2f(z.y, z.x), kRadToDeg), fo, rf, 0u};
}

// ---------------------------------------------------------------------------
// C == 1: the whole spectrum is in this CTA's shared memory.
// ---------------------------------------------------------------------------
SPX_DEV void peaks_single_cta(const float2* s, uint32_t* shist, uint32_t* s_red, const FftGeom& g,
                              uint32_t beam, const FusedArgs& a) {
  const uint32_t tid = threadIdx.x, T = blockDim.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t nw = T >> 5;
  const uint32_t n = a.end > a.start ? a.end - a.start : 0;
  float thr = -INFINITY;
  if (a.factor > 0.0f) {
    for (uint32_t k = a.start + tid; k < a.end; k += T) atomicAdd(&shist[bucket_of(mag_rn(s[sw(k)]))], 1u);
    __syncthreads();
    thr = threshold_from_hist(shist, n, a.factor, s_red);
  }
  const float bw = __fdiv_rn(a.fs, (float)g.nfft);
  if (a.mode == SPX_PEAK_TOPK) {
    // one descending list per warp (lane l holds entry l), merged by warp 0
    uint64_t mine = 0;
    for (uint32_t base = a.start + warp * 32; base < a.end; base += T) {
      const uint32_t k = base + lane;
      uint64_t key = 0;
      bool cand = false;
      if (k < a.end) {
        const float c = mag_rn(s[sw(k)]);
        cand = (c > mag_rn(s[sw(k - 1)])) && (c > mag_rn(s[sw(k + 1)])) && (c > thr);
        key = ((uint64_t)__float_as_uint(c) << 32) | (uint32_t)(~k);
      }
      const uint64_t kth = __shfl_sync(0xffffffffu, mine, a.K - 1);
      uint32_t want = __ballot_sync(0xffffffffu, cand && key > kth);
      while (want) {
        const int src = __ffs(want) - 1;
        want &= want - 1;
        const uint64_t xk = __shfl_sync(0xffffffffu, key, src);
        const uint64_t up = __shfl_up_sync(0xffffffffu, mine, 1);
        if (mine < xk) mine = (lane == 0 || up >= xk) ? xk : up;
      }
    }
    uint64_t* lists = reinterpret_cast<uint64_t*>(shist);  // histogram no longer needed
    __syncthreads();
    lists[warp * 32 + lane] = mine;
    __syncthreads();
    if (warp != 0) return;
    for (uint32_t w = 1; w < nw; ++w) {
      for (uint32_t e = 0; e < a.K; ++e) {
        const uint64_t xk = lists[w * 32 + e];
        if (xk == 0) break;
        const uint64_t up = __shfl_up_sync(0xffffffffu, mine, 1);
        if (mine < xk) mine = (lane == 0 || up >= xk) ? xk : up;
      }
    }
    const uint32_t cnt = __popc(__ballot_sync(0xffffffffu, lane < a.K && mine != 0));
    if (lane == 0) a.counts[beam] = cnt;
    if (lane < cnt) {
      const uint32_t k = ~(uint32_t)mine;
      a.out[(size_t)beam * a.K + lane] =
          fused_max(k, s[sw(k)], mag_rn(s[sw(k - 1)]), __uint_as_float((uint32_t)(mine >> 32)),
                    mag_rn(s[sw(k + 1)]), bw, a.refine);
    }
    return;
  }
  // ALL: ordered compaction over [start, end) in rounds of T consecutive bins.
  uint32_t total = 0;
  for (uint32_t base = a.start; base < a.end; base += T) {
    const uint32_t k = base + tid;
    bool f = false;
    float c = 0.f;
    if (k < a.end) {
      c = mag_rn(s[sw(k)]);
      f = (c > mag_rn(s[sw(k - 1)])) && (c > mag_rn(s[sw(k + 1)])) && (c > thr);
    }
    const uint32_t b = __ballot_sync(0xffffffffu, f);
    if (lane == 0) s_red[warp] = __popc(b);
    __syncthreads();
    uint32_t before = total, all = 0;
    for (uint32_t w = 0; w < nw; ++w) {
      const uint32_t cw = s_red[w];
      if (w < warp) before += cw;
      all += cw;
    }
    if (f) {
      const uint32_t rank = before + __popc(b & ((1u << lane) - 1u));
      if (rank < a.cap)
        a.out[(size_t)beam * a.cap + rank] =
            fused_max(k, s[sw(k)], mag_rn(s[sw(k - 1)]), c, mag_rn(s[sw(k + 1)]), bw, a.refine);
    }
    total += all;
    __syncthreads();
  }
  if (tid == 0) a.counts[beam] = total;
}

// ---------------------------------------------------------------------------
// C > 1: bins k = c + C*i; see the file comment.
// ---------------------------------------------------------------------------
// Exclusive block-wide prefix of one value per thread; returns the prefix and
// writes the total to *total (all threads).  Uses s_red[0..65].
SPX_DEV uint32_t block_exclusive_scan(uint32_t v, uint32_t* s_red, uint32_t* total) {
  const uint32_t tid = threadIdx.x, T = blockDim.x, lane = tid & 31, warp = tid >> 5;
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= (uint32_t)o) x += y;
  }
  if (lane == 31) s_red[warp] = x;
  __syncthreads();
  if (warp == 0) {
    const uint32_t nw = T >> 5;
    uint32_t w = lane < nw ? s_red[lane] : 0u, u = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, u, o);
      if (lane >= (uint32_t)o) u += y;
    }
    if (lane < nw) s_red[32 + lane] = u - w;
    if (lane == nw - 1) s_red[64] = u;
  }
  __syncthreads();
  const uint32_t r = s_red[32 + warp] + x - v;
  *total = s_red[64];
  __syncthreads();
  return r;
}

SPX_DEV void peaks_cluster(float2* s, uint32_t* shist, uint32_t* s_red, uint32_t* shot,
                           uint32_t* slist, uint32_t list_cap, const FftGeom& g, uint32_t c,
                           uint32_t beam, const FusedArgs& a) {
  cg::cluster_group cl = cg::this_cluster();
  const uint32_t tid = threadIdx.x, T = blockDim.x, lane = tid & 31;
  const uint32_t C = g.C, M = g.M;
  const uint32_t n = a.end > a.start ? a.end - a.start : 0;
  const uint32_t i_start = a.start <= c ? 0u : (a.start - c + C - 1) / C;
  const uint32_t i_end = a.end <= c ? 0u : min(M, (a.end - c + C - 1) / C);  // first i with k >= end
  // 1. histogram over [start, end): shared atomics, one global atomic per used bucket.
  //    After the barrier every CTA's spectrum is final, so DSMEM reads are safe
  //    until the last barrier below.
  uint32_t* gh = a.ghist + (size_t)beam * kHist;
  for (uint32_t i = i_start + tid; i < i_end; i += T) atomicAdd(&shist[bucket_of(mag_rn(s[sw(i)]))], 1u);
  __syncthreads();
  for (uint32_t b = tid; b < kHist; b += T)
    if (shist[b]) atomicAdd(&gh[b], shist[b]);
  cl.sync();
  for (uint32_t b = tid; b < kHist; b += T) shist[b] = __ldcg(gh + b);
  __syncthreads();
  const float thr = threshold_from_hist(shist, n, a.factor, s_red);
  // Bins above the threshold's bucket bound the beam's hot bins; the bound
  // is the same in every CTA (same histogram), so the choice below is uniform.
  const uint32_t tb = bucket_of(thr);
  uint32_t hot_bound = 0;
  for (uint32_t b = tid; b < kHist; b += T) hot_bound += b >= tb ? shist[b] : 0u;
  uint32_t hot_total = 0;
  (void)block_exclusive_scan(hot_bound, s_red, &hot_total);
  const bool keep_records = hot_total <= list_cap;
  // 2. classify own hot bins (|X| > thr) against both neighbours, read from
  //    their CTAs; record (i, y_l, y_r) of the maxima for the output.
  auto mag_at = [&](uint32_t k) -> float {
    const uint32_t cc = k % C;
    const float2* src = cc == c ? s : cl.map_shared_rank(s, cc);
    return mag_rn(src[sw(k / C)]);
  };
  const uint32_t words = (M + 31) / 32;
  uint32_t* mywords = shot;  // own maxima bits, bit l of word w <-> i = 32w + l
  float* rec = reinterpret_cast<float*>(slist);  // [list_cap][3] = {i, y_l, y_r}
  uint32_t* s_nrec = s_red + 100;
  for (uint32_t w = tid; w < words; w += T) mywords[w] = 0;
  if (tid == 0) *s_nrec = 0;
  __syncthreads();
  for (uint32_t i = i_start + tid; i < i_end; i += T) {
    const float v = mag_rn(s[sw(i)]);
    if (!(v > thr)) continue;
    const uint32_t k = c + C * i;
    const float yl = mag_at(k - 1), yr = mag_at(k + 1);
    if (v > yl && v > yr) {
      atomicOr(&mywords[i >> 5], 1u << (i & 31));
      if (keep_records) {
        const uint32_t r = atomicAdd(s_nrec, 1u);
        rec[3 * r] = __uint_as_float(i);
        rec[3 * r + 1] = yl;
        rec[3 * r + 2] = yr;
      }
    }
  }
  __syncthreads();
  const size_t beam_words = (size_t)(g.nfft + 31) / 32 + C;
  uint32_t* gm = a.gbits + (size_t)beam * beam_words;  // maxima bitmaps of the cluster
  for (uint32_t w = tid; w < words; w += T) __stcg(gm + (size_t)c * words + w, mywords[w]);
  cl.sync();
  // 3. maxima of the whole beam in bin order, prefix popcount per 1024-bin block
  const uint32_t kwords = (g.nfft + 31) / 32;
  uint32_t* maxbits = shist;
  for (uint32_t w = tid; w < kwords; w += T) maxbits[w] = 0;
  __syncthreads();
  for (uint32_t cw = tid; cw < C * words; cw += T) {
    const uint32_t cc = cw / words, wi = cw % words;
    for (uint32_t t = __ldcg(gm + cw); t; t &= t - 1) {
      const uint32_t k = cc + C * (32 * wi + (__ffs(t) - 1));
      atomicOr(&maxbits[k >> 5], 1u << (k & 31));
    }
  }
  __syncthreads();
  const uint32_t kblocks = (kwords + 31) / 32;  // <= 128
  uint32_t* pref = s_red + 128;
  for (uint32_t blk0 = 0; blk0 < kblocks; blk0 += T / 32) {
    const uint32_t blk = blk0 + (tid >> 5);
    const uint32_t w = blk * 32 + lane;
    uint32_t v = (blk < kblocks && w < kwords) ? __popc(maxbits[w]) : 0u;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0 && blk < kblocks) pref[blk] = v;
  }
  __syncthreads();
  if (tid < 32) {  // exclusive scan of <= 128 block sums, 4 per lane
    uint32_t v[4], sum = 0;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const uint32_t blk = tid * 4 + j;
      v[j] = blk < kblocks ? pref[blk] : 0u;
      sum += v[j];
    }
    uint32_t x = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
      if (tid >= (uint32_t)o) x += y;
    }
    uint32_t run = x - sum;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const uint32_t blk = tid * 4 + j;
      if (blk < kblocks) pref[blk] = run;
      run += v[j];
    }
    if (tid == 31) s_red[64] = x;
  }
  __syncthreads();
  if (c == 0 && tid == 0) a.counts[beam] = s_red[64];
  // 4. own maxima -> MaxValue at their rank
  const float bw = __fdiv_rn(a.fs, (float)g.nfft);
  auto write_max = [&](uint32_t i, float yl, float yr) {
    const uint32_t k = c + C * i;
    uint32_t rank = pref[k >> 10];
    for (uint32_t w2 = (k >> 10) << 5; w2 < (k >> 5); ++w2) rank += __popc(maxbits[w2]);
    rank += __popc(maxbits[k >> 5] & ((1u << (k & 31)) - 1u));
    if (rank < a.cap) {
      const float2 z = s[sw(i)];
      a.out[(size_t)beam * a.cap + rank] = fused_max(k, z, yl, mag_rn(z), yr, bw, a.refine);
    }
  };
  if (keep_records) {
    const uint32_t nrec = *s_nrec;
    for (uint32_t r = tid; r < nrec; r += T)
      write_max(__float_as_uint(rec[3 * r]), rec[3 * r + 1], rec[3 * r + 2]);
    return;  // no DSMEM access after the last barrier
  }
  for (uint32_t w = tid; w < words; w += T)
    for (uint32_t t = mywords[w]; t; t &= t - 1) {
      const uint32_t i = 32 * w + (__ffs(t) - 1), k = c + C * i;
      write_max(i, mag_at(k - 1), mag_at(k + 1));
    }
  cl.sync();  // (many maxima) other CTAs read this CTA's shared memory above
}

template <int EPT>
__global__ void __launch_bounds__(kMaxLocal / EPT, 1)
fft_peaks_kernel(FftGeom g, FusedArgs a) {
  extern __shared__ float2 s[];
  // layout (u32 after the spectrum): histogram / maxima bitmap [4096 + 64] |
  // reductions [256] | own maxima bits [ceil(M/32)] | maxima records [3 * kList]
  uint32_t* shist = reinterpret_cast<uint32_t*>(s + g.Mpad);
  uint32_t* s_red = shist + kHist + 64;
  uint32_t* shot = s_red + 256;
  uint32_t* slist = shot + (g.M + 31) / 32;
  const uint32_t tid = threadIdx.x, T = blockDim.x;
  for (uint32_t b = tid; b < kHist; b += T) shist[b] = 0;
  if (g.C == 1) {
    const uint32_t beam = blockIdx.x;
    prefetch_future_beam(g, a.in, a.n_point, beam, 0, tid, T);
    local_fft<EPT>(s, g, SampleLoader{a.in + (size_t)beam * a.n_point, a.n_point, a.win}, a.tw_local, tid, T);
    peaks_single_cta(s, shist, s_red, g, beam, a);
    return;
  }
  cg::cluster_group cl = cg::this_cluster();
  const uint32_t c = cl.block_rank();
  const uint32_t beam = blockIdx.x / g.C;
  float2* slot = a.xch + (size_t)beam * g.nfft;
  const SampleLoader ld{a.in + (size_t)beam * a.n_point, a.n_point, a.win};
  prefetch_future_beam(g, a.in, a.n_point, beam, c, tid, T);
  switch (g.C) {
    case 2: cross_stage_exchange<2>(slot, c, g.M, ld, a.tw_cross, tid, T); break;
    case 3: cross_stage_exchange<3>(slot, c, g.M, ld, a.tw_cross, tid, T); break;
    case 4: cross_stage_exchange<4>(slot, c, g.M, ld, a.tw_cross, tid, T); break;
    case 6: cross_stage_exchange<6>(slot, c, g.M, ld, a.tw_cross, tid, T); break;
    case 8: cross_stage_exchange<8>(slot, c, g.M, ld, a.tw_cross, tid, T); break;
    case 9: cross_stage_exchange<9>(slot, c, g.M, ld, a.tw_cross, tid, T); break;
    case 12: cross_stage_exchange<12>(slot, c, g.M, ld, a.tw_cross, tid, T); break;
    default: cross_stage_exchange<16>(slot, c, g.M, ld, a.tw_cross, tid, T); break;
  }
  cl.sync();
  const float2* row = slot + (size_t)c * g.M;
  local_fft<EPT>(s, g, ExchangeLoader{row}, a.tw_local, tid, T);
  discard_row_l2(row, (size_t)g.M * sizeof(float2), tid, T);
  peaks_cluster(s, shist, s_red, shot, slist, kList, g, c, beam, a);
}

// Shared memory of the fused kernel for geometry g.
static size_t fused_smem(const FftGeom& g) {
  const size_t hot = g.C > 1 ? (size_t)(g.M + 31) / 32 + 3 * kList : 0;
  return (size_t)g.Mpad * sizeof(float2) + (kHist + 64 + 256 + hot) * sizeof(uint32_t);
}

bool fused_supported(const FftGeom& g, uint32_t mode) {
  if (mode == SPX_PEAK_TOPK) return g.C == 1;
  if (mode != SPX_PEAK_ALL) return false;
  if ((g.nfft + 31) / 32 > kHist) return false;  // maxima bitmap lives in the histogram area
  if ((g.nfft + 31) / 32 > 128 * 32) return false;  // block prefix table holds 128 entries
  return (kHist % g.T) == 0 && g.T <= kList && fused_smem(g) <= 227 * 1024;
}

spx_status launch_fft_peaks(spx_ctx* ctx, const FftPlan& plan, const float2* d_in,
                            uint32_t beams, uint32_t n_point, const float* d_win,
                            uint32_t mode, uint32_t start, uint32_t end, uint32_t cap_or_k,
                            float fs, uint32_t refine, float factor, spx_max_value* d_out,
                            uint32_t* d_counts) {
  if (beams == 0) return SPX_OK;
  FftGeom g = plan.g;
  FusedArgs a{};
  a.in = d_in;
  a.win = d_win;
  a.tw_local = plan.d_tw_local;
  a.tw_cross = plan.d_tw_cross;
  a.out = reinterpret_cast<MaxValueDev*>(d_out);
  a.counts = d_counts;
  a.n_point = n_point;
  a.start = start;
  a.end = end;
  a.mode = mode;
  a.cap = mode == SPX_PEAK_ALL ? cap_or_k : 0;
  a.K = mode == SPX_PEAK_TOPK ? cap_or_k : 0;
  a.refine = refine;
  a.fs = fs;
  a.factor = factor;
  cudaError_t e;
  if (g.C > 1) {
    const size_t xch_bytes = (size_t)beams * g.nfft * sizeof(float2);
    const size_t hist_bytes = (size_t)beams * kHist * sizeof(uint32_t);
    const size_t bits_bytes = (size_t)beams * ((g.nfft + 31) / 32 + g.C) * sizeof(uint32_t);
    void* p = nullptr;
    spx_status st = get_scratch(ctx, kSlotExchange, xch_bytes + hist_bytes + bits_bytes + 512, &p);
    if (st != SPX_OK) return st;
    char* base = static_cast<char*>(p);
    a.xch = reinterpret_cast<float2*>(base);
    a.ghist = reinterpret_cast<uint32_t*>(base + ((xch_bytes + 255) & ~(size_t)255));
    a.gbits = reinterpret_cast<uint32_t*>(reinterpret_cast<char*>(a.ghist) +
                                          ((hist_bytes + 255) & ~(size_t)255));
    e = cudaMemsetAsync(a.ghist, 0, hist_bytes, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaMemsetAsync(histograms)");
  }
  void* args[] = {(void*)&g, (void*)&a};
  const size_t smem = fused_smem(g);
  const void* kfn = g.ept == 32 ? (const void*)fft_peaks_kernel<32> : (const void*)fft_peaks_kernel<16>;
  e = configure_kernel(kfn, 227 * 1024);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "configure fft_peaks_kernel");
  g.beams = beams;
  g.ahead = ctx->input_on_host ? 0u : resident_beams(kfn, g, smem);
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(beams * g.C, 1, 1);
  cfg.blockDim = dim3(g.T, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = ctx->stream;
  cudaLaunchAttribute attr[1];
  if (g.C > 1) {
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = g.C;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
  }
  e = cudaLaunchKernelExC(&cfg, kfn, args);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "launch fft_peaks_kernel");
  return SPX_OK;
}

}  // namespace spx
