// fft_peaks.cu — fused window + zero pad + FFT + |X| + noise threshold +
// peak search from raw samples.  nfft <= 16384: one CTA per beam, the
// spectrum never leaves the chip; larger: see "C > 1" below.
//
// Replaces, for one beam per CTA (nfft <= 16384) or per cluster of C CTAs:
//   PadDataOp + hipfftExecC2C + ComputeMagnitudesOp + AllMaximaPipelineROCm
//   (src/fft_func/src/spectrum_processor_rocm.cpp:444-543,
//    src/fft_func/src/all_maxima_pipeline_rocm.cpp:258-472)
// with the noise threshold and parabolic refinement of this build.
//
// Modes:
//   ALL              : every strict local maximum of |X| in [start, end)
//                      (above the per-beam threshold when one is given),
//                      compacted in bin order.
//   TOPK (C == 1)    : the K largest strict local maxima (optionally above the
//                      threshold), |X| descending, ties by lower bin.
// Results are bit-identical to spx_fft (COMPLEX) followed by spx_all_maxima /
// spx_topk: the same FFT code, |X| = sqrt_rn(re*re + im*im), the same
// histogram-median threshold and the same comparisons.
//
// C > 1 (the beam's bins k = c + C*i are spread over the cluster): the
// cluster FFT writes the bins of the search window into its exchange slot in
// row layout (row c holds X[c + C*i]; the slot's rows are dead by then) and
// maxima_cluster_kernel, one small cluster per beam and several clusters per
// SM, loads |X| of contiguous bin ranges into shared memory, merges their
// noise histograms through distributed shared memory, and classifies and
// ranks the maxima.  Two launches instead of one: the per-beam threshold is a
// dependency across the whole beam, and resolving it inside the FFT cluster
// (one CTA per SM) left the SMs idle on barriers for ~40 % of the launch.
#include <cuda/atomic>

#include "fft_core.cuh"
#include "mlp_device.cuh"
#include "spx_internal.h"

namespace spx {

constexpr uint32_t kHist = 4096;  // noise-histogram buckets (exponent + 4 mantissa bits)

struct FusedArgs {
  const float2* in;
  const float* win;
  const float2* tw_local;
  const float2* tw_cross;
  float2* xch;              // exchange slots (C > 1), one per beam; then the window's bins
  uint32_t* arrive;         // [beams] group-barrier arrivals (C > 1), zeroed by the host
  uint32_t* err;            // device error word
  MaxValueDev* out;
  uint32_t* counts;
  uint32_t n_point, start, end, cap, mode, K, refine;
  float fs, factor;         // factor <= 0: no threshold
  // learned refinement of the top-K peaks (C == 1, mode TOPK): the network's
  // BF16 products and FP32 biases (null: none), amplitude and used flags out
  const __nv_bfloat16* mlp_pb;
  const float* mlp_p;
  float* amp;
  uint32_t* used;
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
// Bin k of the spectrum in shared memory.
struct SmemBins {
  const float2* s;
  SPX_DEV float2 operator()(uint32_t k) const { return s[sw(k)]; }
};

// Shared-memory words the learned refinement needs after the search (it
// reuses the spectrum's): the weights, a 64-float row per warp, then per
// peak a record (8 words), its features and a flag, then the peak count.
constexpr size_t mlp_fused_words(uint32_t warps, uint32_t K) {
  return sizeof(MlpWeights) / 4 + (size_t)warps * kH + (size_t)K * (8 + kIn + 1) + 1;
}

// The learned refinement of the top-K list held by warp 0 (lane l: entry l,
// cnt entries): records and features from the spectrum in shared memory,
// then the weights staged over the spectrum and one warp per peak running
// mlp_forward_warp, with the arithmetic of mlp_refine_kernel.  Every thread
// of the CTA calls it.
__device__ __noinline__ void refine_topk_fused(float2* s, uint64_t mine, const FftGeom& g, uint32_t beam,
                                              const FusedArgs& a, float bw) {
  const uint32_t tid = threadIdx.x, T = blockDim.x, lane = tid & 31, warp = tid >> 5, nw = T >> 5;
  float* base = reinterpret_cast<float*>(s);
  MlpWeights& w = *reinterpret_cast<MlpWeights*>(base);
  float* rows = base + sizeof(MlpWeights) / 4;          // [nw][kH]
  MaxValueDev* rec = reinterpret_cast<MaxValueDev*>(rows + (size_t)nw * kH);  // [K]
  float* feat = reinterpret_cast<float*>(rec + a.K);     // [K][kIn]
  uint32_t* good = reinterpret_cast<uint32_t*>(feat + (size_t)a.K * kIn);  // [K]
  uint32_t& s_cnt = good[a.K];  // (dynamic shared memory: the kernel asks for the 227 KB limit)
  MaxValueDev mv{};
  float fe[kIn];
  bool ok = false;
  uint32_t cnt = 0;
  if (warp == 0) {
    cnt = __popc(__ballot_sync(0xffffffffu, lane < a.K && mine != 0));
    if (lane < cnt) {
      const uint32_t k = ~(uint32_t)mine;
      mv = fused_max(k, s[sw(k)], mag_rn(s[sw(k - 1)]), __uint_as_float((uint32_t)(mine >> 32)),
                     mag_rn(s[sw(k + 1)]), bw, a.refine);
      ok = peak_features_at(SmemBins{s}, a.n_point, g.nfft, k, fe);
    }
  }
  __syncthreads();  // the spectrum is read; its space takes the weights and the peaks
  if (warp == 0) {
    if (lane == 0) {
      s_cnt = cnt;
      a.counts[beam] = cnt;
    }
    if (lane < cnt) {
      rec[lane] = mv;
      for (int i = 0; i < kIn; ++i) feat[(size_t)lane * kIn + i] = fe[i];
      good[lane] = ok ? 1u : 0u;
    }
  }
  mlp_stage(w, a.mlp_pb, a.mlp_p, tid, T);
  __syncthreads();
  cnt = s_cnt;
  for (uint32_t j = warp; j < cnt; j += nw) {
    const bool gd = good[j] != 0;
    float y0 = 0.f, y1 = 0.f;
    if (gd) mlp_forward_warp(w, feat + (size_t)j * kIn, rows + (size_t)warp * kH, lane, &y0, &y1);
    __syncwarp();
    if (lane == 0) {
      MaxValueDev r = rec[j];
      float amp;
      const bool use = mlp_apply(r, gd, y0, y1, a.fs, g.nfft, &amp);
      const size_t idx = (size_t)beam * a.K + j;
      a.out[idx] = r;
      if (a.amp) a.amp[idx] = amp;
      if (a.used) a.used[idx] = use ? 1u : 0u;
    }
  }
}

SPX_DEV void peaks_single_cta(float2* s, uint32_t* shist, uint32_t* s_red, const FftGeom& g,
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
    // one descending list per warp (lane l holds entry l), merged by warp 0;
    // |X| of bins start .. end computed once, neighbours from the next lanes
    uint64_t mine = 0;
    for (uint32_t base = a.start + warp * 32; base < a.end; base += T) {
      const uint32_t k = base + lane;
      const float c = k <= a.end ? mag_rn(s[sw(k)]) : 0.f;
      float lft = __shfl_up_sync(0xffffffffu, c, 1), rgt = __shfl_down_sync(0xffffffffu, c, 1);
      if (lane == 0 && k < a.end) lft = mag_rn(s[sw(k - 1)]);
      if (lane == 31 && k < a.end) rgt = mag_rn(s[sw(k + 1)]);
      const bool cand = k < a.end && c > lft && c > rgt && c > thr;
      const uint64_t key = ((uint64_t)__float_as_uint(c) << 32) | (uint32_t)(~k);
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
    mine = merge_warp_lists(lists, mine, nw, a.K, warp, lane);
    if (a.mlp_pb) return refine_topk_fused(s, mine, g, beam, a, bw);
    if (warp != 0) return;
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
  // ALL: ordered compaction over [start, end) in rounds of T consecutive bins
  // (|X| once per bin, neighbours from the next lanes).
  uint32_t total = 0;
  for (uint32_t base = a.start; base < a.end; base += T) {
    const uint32_t k = base + tid;
    const float c = k <= a.end ? mag_rn(s[sw(k)]) : 0.f;
    float lft = __shfl_up_sync(0xffffffffu, c, 1), rgt = __shfl_down_sync(0xffffffffu, c, 1);
    if (lane == 0 && k < a.end) lft = mag_rn(s[sw(k - 1)]);
    if (lane == 31 && k < a.end) rgt = mag_rn(s[sw(k + 1)]);
    const bool f = k < a.end && c > lft && c > rgt && c > thr;
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
      if (rank < a.cap) a.out[(size_t)beam * a.cap + rank] = fused_max(k, s[sw(k)], lft, c, rgt, bw, a.refine);
    }
    total += all;
    __syncthreads();
  }
  if (tid == 0) a.counts[beam] = total;
}

// ---------------------------------------------------------------------------
// C > 1: the cluster FFT writes the bins of the search window (row layout),
// then maxima_cluster_kernel finds the maxima of each beam.
// ---------------------------------------------------------------------------
// One window of a merged histogram, h[0, W) = buckets b0 .. b0 + W - 1,
// `below` bins lying in lower buckets; r = (n - 1) / 2 is the median rank.
// Computed by one warp (every warp of a CTA may call it; no barrier).  If
// the window holds rank r, *thr = the histogram-interpolated median times
// `factor` (the arithmetic of threshold_from_hist) and returns true;
// *total = the window's bins.
SPX_DEV bool warp_median_window(const uint32_t* h, uint32_t W, uint32_t b0, uint32_t below,
                                uint32_t r, float factor, float* thr, uint32_t* total) {
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t per = (W + 31) / 32;
  const uint32_t lo = min(lane * per, W), hi = min(lo + per, W);
  uint32_t sum = 0;
  for (uint32_t j = lo; j < hi; ++j) sum += h[j];
  uint32_t x = sum;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= (uint32_t)o) x += y;
  }
  *total = __shfl_sync(0xffffffffu, x, 31);
  uint32_t found = 0xFFFFFFFFu, fbelow = 0;
  uint32_t bl = below + x - sum;
  if (bl <= r && r < below + x) {
    for (uint32_t j = lo; j < hi; ++j) {
      const uint32_t cnt = h[j];
      if (bl <= r && r < bl + cnt) {
        found = j;
        fbelow = bl;
        break;
      }
      bl += cnt;
    }
  }
  const uint32_t fl = __ballot_sync(0xffffffffu, found != 0xFFFFFFFFu);
  if (!fl) return false;
  const int src = __ffs(fl) - 1;
  const uint32_t j = __shfl_sync(0xffffffffu, found, src);
  const uint32_t bb = __shfl_sync(0xffffffffu, fbelow, src);
  const uint32_t bk = b0 + j;
  const float flo = __uint_as_float(bk << 19);
  const float fhi = __uint_as_float((bk + 1) << 19);
  const float frac = __fdiv_rn(__fadd_rn((float)(r - bb), 0.5f), (float)h[j]);
  const float med = __fadd_rn(flo, __fmul_rn(__fsub_rn(fhi, flo), frac));
  *thr = __fmul_rn(med, factor);
  return true;
}

// Row c of a beam's exchange slot (read by this CTA alone, dead after its
// local FFT) takes this CTA's bins k = c + C*i in [start - 1, end + 1) (the
// search window and the neighbours of its end bins): row[i] = X[c + C*i].
// The rest of the row is discarded from L2.
struct WindowRows {
  uint32_t ilo, ihi;  // row indices i of the CTA's window bins: [ilo, ihi)
};
SPX_DEV WindowRows window_rows(const FftGeom& g, uint32_t c, uint32_t start, uint32_t end) {
  const uint32_t klo = start - 1, khi = min(end + 1, g.nfft);
  const uint32_t ilo = klo <= c ? 0u : (klo - c + g.C - 1) / g.C;
  const uint32_t ihi = khi <= c ? 0u : min(g.M, (khi - c + g.C - 1) / g.C);
  return WindowRows{ilo, ihi};
}

// Drops from L2, without write-back, the lines of the row outside the window.
SPX_DEV void discard_outside_window(float2* row, const FftGeom& g, WindowRows w, uint32_t tid, uint32_t T) {
  if (w.ihi > w.ilo) {
    discard_row_l2(row, (size_t)w.ilo * sizeof(float2), tid, T);
    discard_row_l2(row + w.ihi, (size_t)(g.M - w.ihi) * sizeof(float2), tid, T);
  } else {
    discard_row_l2(row, (size_t)g.M * sizeof(float2), tid, T);
  }
}

SPX_DEV void write_window_row(float2* row, const float2* s, const FftGeom& g, uint32_t c, uint32_t start,
                              uint32_t end, uint32_t tid, uint32_t T) {
  const WindowRows w = window_rows(g, c, start, end);
  for (uint32_t i = w.ilo + tid; i < w.ihi; i += T) __stcg(row + i, s[sw(i)]);
  discard_outside_window(row, g, w, tid, T);
}

// Output of the last local pass straight into the window part of the row.
struct WindowRowOut {
  float2* row;
  WindowRows w;
  SPX_DEV void operator()(uint32_t i, float2 z) const {
    if (i >= w.ilo && i < w.ihi) __stcg(row + i, z);
  }
};

template <int EPT>
__global__ void __launch_bounds__(kMaxLocal / EPT, 1)
fft_peaks_kernel(FftGeom g, FusedArgs a) {
  extern __shared__ float2 s[];
  // C == 1, after the spectrum: histogram (with a threshold) or top-K lists
  // [fused_extra_words - 256] | reductions [256]
  const uint32_t tid = threadIdx.x, T = blockDim.x;
  uint32_t* shist = reinterpret_cast<uint32_t*>(s + g.Mpad);
  uint32_t* s_red = shist + (a.factor > 0.0f ? kHist + 64 : 2 * T);
  if (g.C == 1) {
    if (a.factor > 0.0f)
      for (uint32_t b = tid; b < kHist; b += T) shist[b] = 0;
    const uint32_t beam = blockIdx.x;
    prefetch_future_beam(g, a.in, a.n_point, beam, 0, tid, T);
    local_fft<EPT>(s, g, SampleLoader{a.in + (size_t)beam * a.n_point, a.n_point, a.win}, a.tw_local, tid, T);
    peaks_single_cta(s, shist, s_red, g, beam, a);
    return;
  }
  // C > 1 (sizes fft_group_kernel does not take): one cluster per beam
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
  float2* row = slot + (size_t)c * g.M;
  local_fft<EPT>(s, g, ExchangeLoader{row}, a.tw_local, tid, T);
  write_window_row(row, s, g, c, a.start, a.end, tid, T);
}

// C > 1 with a power-of-two local size M (4096, 8192, 16384; M / 16 threads)
// and C in {2, 4, 8, 16}: a persistent cooperative launch of G groups of C
// CTAs (one CTA per SM); group q transforms beams q, q + G, ...  Per beam:
// the cross stage into the beam's exchange slot, a group barrier, the local
// FFT of row c, the window's bins into row c.  Clusters of 8 one-SM CTAs
// fit on 120 of the 152 SMs; groups use all of them.
template <int M>
__global__ void __launch_bounds__(M / 16, 16384 / M)
fft_group_kernel(FftGeom g, FusedArgs a, uint32_t groups) {
  extern __shared__ float2 s[];
  constexpr uint32_t T = M / 16;
  const uint32_t tid = threadIdx.x;
  const uint32_t grp = blockIdx.x / g.C, c = blockIdx.x - grp * g.C;
  // cross stage of a beam into its exchange slot, then this CTA's arrival
  auto cross = [&](uint32_t beam) {
    float2* slot = a.xch + (size_t)beam * g.nfft;
    const SampleLoader ld{a.in + (size_t)beam * a.n_point, a.n_point, a.win};
    prefetch_future_beam(g, a.in, a.n_point, beam, c, tid, T);
    switch (g.C) {
      case 2: cross_stage_exchange<2>(slot, c, M, ld, a.tw_cross, tid, T); break;
      case 4: cross_stage_exchange<4>(slot, c, M, ld, a.tw_cross, tid, T); break;
      case 8: cross_stage_exchange<8>(slot, c, M, ld, a.tw_cross, tid, T); break;
      default: cross_stage_exchange<16>(slot, c, M, ld, a.tw_cross, tid, T); break;
    }
    group_arrive(a.arrive + beam);
  };
  // The cross stage of the group's next beam runs between the arrival and
  // the wait of the current one: a CTA that waits for its group's slowest
  // member does so with the next beam's samples already exchanged.
  if (grp < g.beams) cross(grp);
#pragma unroll 1
  for (uint32_t beam = grp; beam < g.beams; beam += groups) {
    if (beam + groups < g.beams) cross(beam + groups);
    group_wait(a.arrive + beam, g.C, a.err);
    float2* row = a.xch + (size_t)beam * g.nfft + (size_t)c * M;
    // the last pass writes the window's bins of the row straight from its
    // registers (no store to shared memory, barrier and reload)
    const WindowRows w = window_rows(g, c, a.start, a.end);
    ct_local_fft_out<M>(s, ExchangeLoader{row}, a.tw_local, tid, WindowRowOut{row, w});
    discard_outside_window(row, g, w, tid, T);
  }  // (the next beam's group_arrive barrier orders these reads of s before its first pass)
}

// Self-test of the bounded wait: a single CTA arrives at a barrier that
// expects two arrivals, so the wait ends at its time bound.
__global__ void group_timeout_probe_kernel(uint32_t* count, uint32_t* err) { group_barrier(count, 2u, err); }

spx_status launch_group_timeout_probe(spx_ctx* ctx, uint32_t* d_count) {
  cudaError_t e = cudaMemsetAsync(d_count, 0, sizeof(uint32_t), ctx->stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "group probe memset");
  group_timeout_probe_kernel<<<1, 32, 0, ctx->stream>>>(d_count, ctx->d_error);
  e = cudaGetLastError();
  return e == cudaSuccess ? SPX_OK : cuda_fail(ctx, e, "launch group_timeout_probe_kernel");
}


// ---------------------------------------------------------------------------
// maxima_cluster_kernel: every strict local maximum of |X| in [start, end)
// above the per-beam threshold, compacted in bin order.  A cluster of C2
// CTAs per beam; CTA c owns bins [start + c*chunk, start + (c+1)*chunk) and
// keeps their |X| in shared memory:
//  1. |X| of the CTA's bins and both neighbours of its range; with a
//     threshold, a local histogram and its bucket range;
//  2. (threshold) cluster barrier; the merged histogram over the union of the
//     bucket ranges, read from every CTA through distributed shared memory;
//     the threshold computed per warp;
//  3. maxima flags (a bitmap in bin order) and their number, published in
//     device memory; cluster barrier;
//  4. rank of a maximum = maxima of the lower CTAs + maxima before it in
//     this CTA; records written for ranks below the capacity.
// The spectrum of beam b holds bin k at spec[b*nfft + (k mod C1)*M1 + k div C1]
// (C1 = 1: natural order; C1 > 1: the cluster FFT's row layout).
// ---------------------------------------------------------------------------
constexpr uint32_t kMxThreads = 256;
constexpr uint32_t kMxMinBlocks = 5;  // CTAs per SM the kernel is built for (<= 48 registers)
constexpr uint32_t kMxMaxC2 = 8;
constexpr uint32_t kMxMaxChunk = 32768;  // < 65536: 16-bit histogram counters cannot overflow
constexpr uint32_t kMxBatch = 4;         // loads in flight per thread (8 and 16 measured slower)
static_assert(kMxMaxC2 * kMxMaxChunk == kMaxClusterSpan, "window limit of spx_all_maxima");
constexpr uint32_t kMxMerge = 512;       // buckets of the merged histogram per window

struct MxArgs {
  const float2* spec;
  uint32_t* ccount;      // [beams][C2] maxima per CTA (scratch)
  MaxValueDev* out;
  uint32_t* counts;
  uint32_t C1, M1;
  uint32_t c1shift;      // log2(C1) when C1 is a power of two, else 32
  uint32_t c1magic;      // ceil(2^32 / C1) (C1 not a power of two)
  uint32_t nfft, start, end, cap, refine, chunk;
  float fs, factor;      // factor <= 0: no threshold
};

// Bin k of a beam's spectrum (offsets < nfft <= 2^21 fit 32 bits).
SPX_DEV float2 mx_load(const MxArgs& a, const float2* __restrict__ sb, uint32_t k) {
  uint32_t q, r;
  if (a.c1shift < 32) {
    q = k >> a.c1shift;
    r = k & (a.C1 - 1);
  } else {
    q = __umulhi(k, a.c1magic);  // k div C1 (exact: k * C1 < 2^32)
    r = k - q * a.C1;
  }
  return __ldcs(sb + (r * a.M1 + q));
}

// Shared memory (32-bit words): |X| [chunk + 2] | maxima bits [chunk/32] |
// reductions [64] | with a threshold: 16-bit histogram [kHist/2] | merged
// window [kMxMerge].
static size_t mx_smem_words(uint32_t chunk, bool thr) {
  return (size_t)chunk + 2 + (chunk + 31) / 32 + 64 + (thr ? kHist / 2 + kMxMerge : 0);
}

__global__ void __launch_bounds__(kMxThreads, kMxMinBlocks)
maxima_cluster_kernel(MxArgs a) {
  extern __shared__ uint32_t smx[];
  cg::cluster_group cl = cg::this_cluster();
  const uint32_t C2 = cl.num_blocks(), c = cl.block_rank(), beam = blockIdx.x / C2;
  const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const bool thr_on = a.factor > 0.0f;
  float* smag = reinterpret_cast<float*>(smx);         // [chunk + 2]: bins lo - 1 .. hi
  uint32_t* bits = smx + a.chunk + 2;                   // [chunk / 32]
  uint32_t* red = bits + (a.chunk + 31) / 32;           // [64]
  uint32_t* hist = red + 64;                            // [kHist / 2]: bucket b in half b & 1 of word b / 2
  uint32_t* merged = hist + kHist / 2;                  // [kMxMerge]
  const uint32_t lo = min(a.start + c * a.chunk, a.end);
  const uint32_t hi = min(lo + a.chunk, a.end);
  const uint32_t nb = hi - lo;
  const float2* sb = a.spec + (size_t)beam * a.nfft;
  if (thr_on) {
    for (uint32_t b = tid; b < kHist / 2; b += kMxThreads) hist[b] = 0;
    if (tid == 0) {
      red[0] = kHist;
      red[1] = 0;
    }
    __syncthreads();
  }
  // 1. (loads issued kMxBatch at a time per thread, so that enough bytes
  //    are in flight to cover the device-memory latency)
  uint32_t bmin = kHist, bmax = 0;
  if (nb && tid < 2) smag[tid ? nb + 1 : 0] = mag_rn(mx_load(a, sb, tid ? hi : lo - 1));  // neighbours
  auto take = [&](uint32_t i, float2 z) {  // |X| of bin lo + i into shared memory and the histogram
    const float m = mag_rn(z);
    smag[i + 1] = m;
    if (thr_on) {
      const uint32_t b = bucket_of(m);
      atomicAdd(&hist[b >> 1], 1u << ((b & 1u) * 16));
      bmin = min(bmin, b);
      bmax = max(bmax, b);
    }
  };
  // Power-of-two C1 divides kMxThreads: the kMxBatch bins lo + i0 + j*256 + tid
  // of a full batch lie in one row, 256 / C1 columns apart.
  const bool rows_fixed = a.c1shift < 32;
  for (uint32_t i0 = 0; i0 < nb; i0 += kMxBatch * kMxThreads) {
    float2 z[kMxBatch];
    if (rows_fixed && i0 + kMxBatch * kMxThreads <= nb) {
      const uint32_t k = lo + i0 + tid;
      const float2* p = sb + ((k & (a.C1 - 1)) * a.M1 + (k >> a.c1shift));
      const uint32_t step = kMxThreads >> a.c1shift;
#pragma unroll
      for (uint32_t j = 0; j < kMxBatch; ++j) z[j] = __ldcs(p + j * step);
#pragma unroll
      for (uint32_t j = 0; j < kMxBatch; ++j) take(i0 + j * kMxThreads + tid, z[j]);
      continue;
    }
#pragma unroll
    for (uint32_t j = 0; j < kMxBatch; ++j) {
      const uint32_t i = i0 + j * kMxThreads + tid;
      if (i < nb) z[j] = mx_load(a, sb, lo + i);
    }
#pragma unroll
    for (uint32_t j = 0; j < kMxBatch; ++j) {
      const uint32_t i = i0 + j * kMxThreads + tid;
      if (i < nb) take(i, z[j]);
    }
  }
  float thr = -INFINITY;
  if (thr_on) {
    bmin = __reduce_min_sync(0xffffffffu, bmin);
    bmax = __reduce_max_sync(0xffffffffu, bmax);
    if (lane == 0 && bmin <= bmax) {
      atomicMin(&red[0], bmin);
      atomicMax(&red[1], bmax);
    }
    __syncthreads();
    cl.sync();  // every histogram complete; read remotely until the next cluster barrier
    // 2.
    if (warp == 0) {
      uint32_t l = kHist, h = 0;
      if (lane < C2) {
        const uint32_t* r = cl.map_shared_rank(red, lane);
        l = r[0];
        h = r[1];
      }
      l = __reduce_min_sync(0xffffffffu, l);
      h = __reduce_max_sync(0xffffffffu, h);
      if (lane == 0) {
        red[2] = l;
        red[3] = h;
      }
    }
    __syncthreads();
    const uint32_t b0 = red[2];
    const uint32_t R = b0 <= red[3] ? red[3] - b0 + 1 : 0u;
    const uint32_t n = a.end > a.start ? a.end - a.start : 0u;
    thr = INFINITY;
    // the merged histogram in windows of kMxMerge buckets (one window unless
    // |X| spans more than 2^(kMxMerge/16) in ratio); same steps in every CTA
    uint32_t below = 0;
    for (uint32_t w0 = 0; n > 0 && w0 < R; w0 += kMxMerge) {
      const uint32_t W = min(kMxMerge, R - w0);
      for (uint32_t t = tid; t < W; t += kMxThreads) {
        const uint32_t b = b0 + w0 + t;
        uint32_t sum = 0;
#pragma unroll
        for (uint32_t cc = 0; cc < kMxMaxC2; ++cc)
          if (cc < C2) sum += (cl.map_shared_rank(hist, cc)[b >> 1] >> ((b & 1u) * 16)) & 0xFFFFu;
        merged[t] = sum;
      }
      __syncthreads();
      uint32_t wtot = 0;
      const bool done = warp_median_window(merged, W, b0 + w0, below, (n - 1) / 2, a.factor, &thr, &wtot);
      __syncthreads();  // merged rewritten by the next window
      if (done) break;
      below += wtot;
    }
  } else {
    __syncthreads();
  }
  // 3. a thread tests 4 consecutive bins i = 4*(u*256 + tid) .. +3 from one
  //    16-byte and one 8-byte load of |X| (bin i is smag[i + 1]); the 8
  //    lanes of a group of 32 bins merge their 4-bit pieces into the word.
  const uint32_t words = (nb + 31) / 32;
  for (uint32_t u = 0; u * 4 * kMxThreads < nb; ++u) {
    const uint32_t i = 4 * (u * kMxThreads + tid);
    uint32_t piece = 0;
    if (i < nb) {  // smag[i .. i + 5]: i + 5 <= chunk + 1, inside the array
      const float4 m4 = *reinterpret_cast<const float4*>(smag + i);
      const float2 m2 = *reinterpret_cast<const float2*>(smag + i + 4);
      const float m[6] = {m4.x, m4.y, m4.z, m4.w, m2.x, m2.y};
#pragma unroll
      for (int j = 0; j < 4; ++j)
        if (i + j < nb && m[j + 1] > m[j] && m[j + 1] > m[j + 2] && m[j + 1] > thr) piece |= 1u << j;
    }
    uint32_t word = piece << (4 * (lane & 7));
    word |= __shfl_xor_sync(0xffffffffu, word, 1);
    word |= __shfl_xor_sync(0xffffffffu, word, 2);
    word |= __shfl_xor_sync(0xffffffffu, word, 4);
    const uint32_t w = u * (4 * kMxThreads / 32) + warp * 4 + (lane >> 3);
    if ((lane & 7) == 0 && w < words) bits[w] = word;
  }
  __syncthreads();
  // contiguous words per thread, block-wide exclusive scan of their maxima
  const uint32_t per = (words + kMxThreads - 1) / kMxThreads;
  const uint32_t w0 = min(tid * per, words), w1 = min(w0 + per, words);
  uint32_t mine = 0;
  for (uint32_t w = w0; w < w1; ++w) mine += __popc(bits[w]);
  uint32_t x = mine;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= (uint32_t)o) x += y;
  }
  if (lane == 31) red[8 + warp] = x;
  __syncthreads();
  uint32_t before = 0, own = 0;
#pragma unroll
  for (uint32_t w = 0; w < kMxThreads / 32; ++w) {
    const uint32_t v = red[8 + w];
    before += w < warp ? v : 0u;
    own += v;
  }
  uint32_t rank = before + x - mine;
  uint32_t* cc_counts = a.ccount + (size_t)beam * C2;
  if (C2 > 1) {
    if (tid == 0) __stcg(cc_counts + c, own);
    cl.sync();  // counts visible; no distributed shared memory access after this barrier
  }
  uint32_t base = 0, total = own;
  if (C2 > 1) {
    total = 0;
    for (uint32_t cc = 0; cc < C2; ++cc) {
      const uint32_t v = __ldcg(cc_counts + cc);
      base += cc < c ? v : 0u;
      total += v;
    }
  }
  if (c == 0 && tid == 0) a.counts[beam] = total;
  // 4.
  rank += base;
  if (rank >= a.cap) return;
  const float bw = __fdiv_rn(a.fs, (float)a.nfft);
  MaxValueDev* o = a.out + (size_t)beam * a.cap;
  for (uint32_t w = w0; w < w1 && rank < a.cap; ++w) {
    for (uint32_t t = bits[w]; t && rank < a.cap; t &= t - 1) {
      const uint32_t i = 32 * w + (__ffs(t) - 1), k = lo + i;
      o[rank++] = fused_max(k, mx_load(a, sb, k), smag[i], smag[i + 1], smag[i + 2], bw, a.refine);
    }
  }
}

// Shared memory of the fused kernel for geometry g: after the spectrum, with
// a noise threshold the histogram (kHist + 64 words), else the top-K lists (a
// 64-bit entry per thread), then 256 words of reductions.  Without the
// threshold's 16 KB, an 8192-point beam's CTA fits three to an SM.
static size_t fused_smem(const FftGeom& g, bool threshold = true) {
  if (g.C != 1) return (size_t)g.Mpad * sizeof(float2);
  return (size_t)g.Mpad * sizeof(float2) + ((threshold ? kHist + 64 : 2 * g.T) + 256) * sizeof(uint32_t);
}

// Cluster size and bins per CTA of maxima_cluster_kernel for a window of `span` bins.
static bool mx_geometry(uint32_t span, uint32_t* C2, uint32_t* chunk) {
  uint32_t c2 = (span + 8191) / 8192;
  if (c2 < 1) c2 = 1;
  if (c2 > kMxMaxC2) c2 = kMxMaxC2;
  uint32_t ch = (span + c2 - 1) / c2;
  ch = (ch + 31) & ~31u;
  if (ch == 0) ch = 32;
  if (ch > kMxMaxChunk) return false;
  *C2 = c2;
  *chunk = ch;
  return true;
}

bool fused_mlp_supported(const FftGeom& g, uint32_t K) {
  return g.C == 1 && fused_supported(g, SPX_PEAK_TOPK) && K >= 1 && K <= 32 &&
         2 * (size_t)g.Mpad >= mlp_fused_words(g.T / 32, K);
}

bool fused_supported(const FftGeom& g, uint32_t mode) {
  if (mode != SPX_PEAK_ALL && mode != SPX_PEAK_TOPK) return false;
  if (g.C == 1) return (kHist % g.T) == 0 && fused_smem(g) <= 227 * 1024;
  if (mode == SPX_PEAK_TOPK) return false;
  uint32_t c2, ch;
  return mx_geometry(g.nfft, &c2, &ch) && g.C <= 16;
}

spx_status launch_maxima_cluster(spx_ctx* ctx, const float2* d_spec, uint32_t C1, uint32_t M1,
                                 uint32_t beams, uint32_t nfft, uint32_t start, uint32_t end,
                                 uint32_t cap, float fs, uint32_t refine, float factor,
                                 uint32_t* d_ccount, spx_max_value* d_out, uint32_t* d_counts) {
  if (beams == 0) return SPX_OK;
  uint32_t C2 = 1, chunk = 32;
  if (!mx_geometry(end > start ? end - start : 0u, &C2, &chunk))
    return fail(ctx, SPX_ERR_INVALID_ARG, "maxima: search window too long");
  MxArgs a{};
  a.spec = d_spec;
  a.ccount = d_ccount;
  a.out = reinterpret_cast<MaxValueDev*>(d_out);
  a.counts = d_counts;
  a.C1 = C1;
  a.M1 = M1;
  a.c1shift = (C1 & (C1 - 1)) == 0 ? (uint32_t)__builtin_ctz(C1) : 32u;
  a.c1magic = a.c1shift == 32 ? (uint32_t)(((1ull << 32) + C1 - 1) / C1) : 0u;
  a.nfft = nfft;
  a.start = start;
  a.end = end;
  a.cap = cap;
  a.refine = refine;
  a.chunk = chunk;
  a.fs = fs;
  a.factor = factor;
  const size_t smem = mx_smem_words(chunk, factor > 0.0f) * sizeof(uint32_t);
  cudaError_t e = configure_kernel((const void*)maxima_cluster_kernel, 227 * 1024);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "configure maxima_cluster_kernel");
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(beams * C2, 1, 1);
  cfg.blockDim = dim3(kMxThreads, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = ctx->stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = C2;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  e = cudaLaunchKernelEx(&cfg, maxima_cluster_kernel, a);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "launch maxima_cluster_kernel");
  return SPX_OK;
}

spx_status launch_fft_peaks(spx_ctx* ctx, const FftPlan& plan, const float2* d_in,
                            uint32_t beams, uint32_t n_point, const float* d_win,
                            uint32_t mode, uint32_t start, uint32_t end, uint32_t cap_or_k,
                            float fs, uint32_t refine, float factor, spx_max_value* d_out,
                            uint32_t* d_counts, const MlpRefineArgs* mlp) {
  if (beams == 0) return SPX_OK;
  FftGeom g = plan.g;
  FusedArgs a{};
  if (mlp) {
    a.mlp_pb = static_cast<const __nv_bfloat16*>(mlp->pb);
    a.mlp_p = mlp->p;
    a.amp = mlp->amp;
    a.used = mlp->used;
  }
  a.in = d_in;
  a.win = d_win;
  a.tw_local = plan.d_tw_local;
  a.tw_cross = plan.d_tw_cross;
  a.out = reinterpret_cast<MaxValueDev*>(d_out);
  a.counts = d_counts;
  a.err = ctx->d_error;
  a.n_point = n_point;
  a.start = start;
  a.end = end;
  a.mode = mode;
  a.cap = mode == SPX_PEAK_ALL ? cap_or_k : 0;
  a.K = mode == SPX_PEAK_TOPK ? cap_or_k : 0;
  a.refine = refine;
  a.fs = fs;
  a.factor = factor;
  const size_t smem = fused_smem(g, factor > 0.0f);
  g.beams = beams;
  cudaError_t e;
  if (g.C == 1) {
    const void* kfn = g.ept == 32 ? (const void*)fft_peaks_kernel<32> : (const void*)fft_peaks_kernel<16>;
    e = configure_kernel(kfn, 227 * 1024);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "configure fft_peaks_kernel");
    g.ahead = ctx->input_on_host ? 0u : resident_beams(kfn, g, smem);
    void* args[] = {(void*)&g, (void*)&a};
    e = cudaLaunchKernel(kfn, dim3(beams), dim3(g.T), args, smem, ctx->stream);
    return e == cudaSuccess ? SPX_OK : cuda_fail(ctx, e, "launch fft_peaks_kernel");
  }
  // C > 1: scratch = exchange slots | per-CTA maxima counts | group-barrier arrivals
  const size_t xch_bytes = ((size_t)beams * g.nfft * sizeof(float2) + 255) & ~(size_t)255;
  const size_t cnt_bytes = ((size_t)beams * kMxMaxC2 * sizeof(uint32_t) + 255) & ~(size_t)255;
  void* p = nullptr;
  spx_status st = get_scratch(ctx, kSlotExchange, xch_bytes + cnt_bytes + (size_t)beams * sizeof(uint32_t), &p);
  if (st != SPX_OK) return st;
  a.xch = static_cast<float2*>(p);
  uint32_t* ccount = reinterpret_cast<uint32_t*>(static_cast<char*>(p) + xch_bytes);
  a.arrive = reinterpret_cast<uint32_t*>(static_cast<char*>(p) + xch_bytes + cnt_bytes);
  if (group_geometry(g)) {
    e = cudaMemsetAsync(a.arrive, 0, (size_t)beams * sizeof(uint32_t), ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaMemsetAsync(group barriers)");
    const void* kfn = g.M == 16384 ? (const void*)fft_group_kernel<16384>
                      : g.M == 8192 ? (const void*)fft_group_kernel<8192>
                                    : (const void*)fft_group_kernel<4096>;
    e = configure_kernel(kfn, 227 * 1024);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "configure fft_group_kernel");
    // as many groups as can be resident at once (cooperative launch), at most one per beam
    uint32_t groups = resident_ctas(kfn, g.T, smem, 1) / g.C;
    if (groups > beams) groups = beams;
    if (groups == 0) return fail(ctx, SPX_ERR_CUDA, "fft_group_kernel: a group of CTAs does not fit the device");
    // prefetch distance: one round of the groups (also for samples in host
    // memory, which then cross the host link while the current beams compute)
    g.ahead = groups;
    void* args[] = {(void*)&g, (void*)&a, (void*)&groups};
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(groups * g.C, 1, 1);
    cfg.blockDim = dim3(g.T, 1, 1);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = ctx->stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    e = cudaLaunchKernelExC(&cfg, kfn, args);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "launch fft_group_kernel");
  } else {
    const void* kfn = g.ept == 32 ? (const void*)fft_peaks_kernel<32> : (const void*)fft_peaks_kernel<16>;
    e = configure_kernel(kfn, 227 * 1024);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "configure fft_peaks_kernel");
    g.ahead = ctx->input_on_host ? 0u : resident_beams(kfn, g, smem);
    void* args[] = {(void*)&g, (void*)&a};
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(beams * g.C, 1, 1);
    cfg.blockDim = dim3(g.T, 1, 1);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = ctx->stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = g.C;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    e = cudaLaunchKernelExC(&cfg, kfn, args);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "launch fft_peaks_kernel");
  }
  return launch_maxima_cluster(ctx, a.xch, g.C, g.M, beams, g.nfft, start, end, cap_or_k, fs, refine,
                               factor, ccount, d_out, d_counts);
}

}  // namespace spx
