// batch.cu — many beams of uneven length and FFT size in one launch.
//
// A batch holds, for B beams with their own n_point and nfft (2^a*3^b), the
// per-size FFT plans, the packing of all beams into the clusters of a single
// launch, the device scratch (exchange slots) and optionally a CUDA graph of
// a run.  A run is two launches:
//   1. fft_batch_kernel: every beam's windowed, zero-padded FFT in ONE
//      launch.  Beam b with nfft = C x M takes C CTAs (ranks 0..C-1) of one
//      cluster; a cluster of Cl CTAs (Cl = the largest C, or more, chosen
//      by spx_batch_set_cluster or the autotuner) hosts one or
//      several beams on disjoint rank ranges (first-fit decreasing, largest
//      beams first).  A CTA runs the cross stage of its rank (C > 1: the
//      C-point DFTs of its columns, window and zero padding on load, into the
//      beam's exchange slot; C = 1: the windowed, zero-padded samples), the
//      cluster barrier, then the M-point local FFT of its row in shared
//      memory (compile-time plans for the sizes of ct_menu_fft, the runtime
//      plan otherwise), and leaves the row in the slot (row c: X[c + C*i]).
//      It also prefetches into L2 the samples of the CTA one residency wave
//      later.
//   2. topk_batch_kernel: the K largest strict local maxima of every beam,
//      one CTA per beam, reading bin k from row k mod C of the beam's slot.
// The plans are the context's plans for those sizes and the window is
// evaluated by window_at (the function that fills spx_fft's tables): every
// beam's list is the bits of spx_fft_peaks on that beam alone.
// spx_batch_run_per_size runs the same kernels once per distinct nfft.
//
// Measured on GB300 and not kept (uneven workload, 1024 beams):
//  * a persistent cooperative kernel over a queue of (beam, rank) slots: the
//    compile-time FFTs of many sizes cannot stay in registers inside a loop
//    (out-of-line calls spill 200-500 bytes per thread, inlined sizes
//    more): 1.10 ms per step, ~950 MB of spill traffic through L1;
//  * the top-K fused into the FFT launch (the last CTA of a beam to finish
//    its row scans the beam): 1.33 ms against 0.81 ms for the FFT launch
//    alone: that CTA holds its SM through the scan, and clusters only start
//    where a GPC has Cl free SMs.
//
// No reference counterpart: DspSpectrum transforms one size per call
// (FFTProcessorROCm, hipfftPlan1d with one nFFT per plan,
// src/fft_func/src/fft_processor_rocm.cpp:152-193); its nearest piece is host
// batching (BatchManager, src/fft_func/src/spectrum_processor_rocm.cpp:289-304).
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <fstream>
#include <functional>
#include <map>
#include <sstream>
#include <vector>

#include "fft_core.cuh"
#include "spx_internal.h"

namespace spx {

struct BatchBeam {
  uint64_t in_off;    // first sample in the packed input (complex elements)
  uint64_t spec_off;  // first element of the beam's exchange slot (its spectrum rows after the FFT)
  uint32_t n_point, nfft, geom, pad;
};
constexpr uint32_t kIdle = 0xFFFFFFFFu;
struct BatchCta {
  uint32_t beam;  // kIdle: this CTA has no work
  uint32_t c;     // rank within the beam's CTAs
};
struct BatchGeom {
  FftGeom g;
  const float2* twl;
  const float2* twc;
};

constexpr uint32_t kBpThreads = 1024;  // threads of a batch CTA (16 points each at M = 16384)
constexpr uint32_t kBtMaxC = 16;       // CTAs per beam
constexpr size_t kBpFftBytes = (size_t)sw_len(kMaxLocal) * sizeof(float2);
constexpr size_t kBpSmem = kBpFftBytes;
constexpr uint32_t kBtThreads = 256;  // threads of a top-K CTA (one beam)

// Peak-search parameters and outputs of a batch.
struct TopkArgs {
  MaxValueDev* out;
  uint32_t* counts;
  uint32_t K, start, end, refine;
  float fs;
};

struct BatchArgs {
  const float2* in;
  const BatchBeam* beams;
  const BatchGeom* geoms;
  const BatchCta* ctas;
  uint32_t window;
  uint32_t ahead;  // CTAs of one residency wave (L2 prefetch distance; 0: none)
  float2* xch;
};

// Sample n of one beam of the batch: the window evaluated per sample by
// window_at (the function that fills the per-size kernels' window tables, so
// a batched beam and the same beam through spx_fft get the same windowed
// bits), zero beyond n_point.
struct SampleLoaderOTF {
  const float2* __restrict__ x;
  uint32_t n_point;
  WindowGen wg;
  SPX_DEV float2 operator()(uint32_t n) const {
    float2 a = make_float2(0.f, 0.f);
    if (n < n_point) {
      a = ld_stream(x + n);
      if (wg.kind != SPX_WINDOW_NONE) {
        const float w = window_at(wg, n);
        a.x = __fmul_rn(a.x, w);
        a.y = __fmul_rn(a.y, w);
      }
    }
    return a;
  }
};

template <int CR>
SPX_DEV void cross_otf(float2* slot, uint32_t c, uint32_t M, const SampleLoaderOTF& ld,
                       const float2* twc, uint32_t tid) {
  const uint32_t S = (M + CR - 1) / CR;
  const uint32_t lo = c * S, hi = min(lo + S, M);
#pragma unroll 2
  for (uint32_t n2 = lo + tid; n2 < hi; n2 += kBpThreads) {
    float2 v[CR];
#pragma unroll
    for (int n1 = 0; n1 < CR; ++n1) v[n1] = ld(n1 * M + n2);
    Dft<CR>::run(v);
    __stcg(slot + n2, v[0]);
    // W_N^{n2 k1} by the product tree of cross_stage_exchange
    float2 w[CR];
    w[1] = __ldg(twc + n2);
#pragma unroll
    for (int k1 = 2; k1 < CR; ++k1) w[k1] = (k1 % 2 == 0) ? cmul(w[k1 / 2], w[k1 / 2]) : cmul(w[k1 - 1], w[1]);
#pragma unroll
    for (int k1 = 1; k1 < CR; ++k1) __stcg(slot + (size_t)k1 * M + n2, cmul(v[k1], w[k1]));
  }
}

// Preparation of slot (b, c): the cross stage of rank c (C > 1) or the
// windowed, zero-padded samples (C = 1), into the beam's exchange slot.
__device__ __noinline__ void bp_prepare(const FftGeom* g, float2* slot, uint32_t c, const float2* x,
                                        uint32_t n_point, uint32_t window, const float2* twc) {
  const uint32_t tid = threadIdx.x, M = g->M;
  const SampleLoaderOTF ld{x, n_point, make_window_gen(window, n_point)};
  switch (g->C) {
    case 1:
      for (uint32_t n = tid; n < M; n += kBpThreads) __stcg(slot + n, ld(n));
      break;
    case 2: cross_otf<2>(slot, c, M, ld, twc, tid); break;
    case 3: cross_otf<3>(slot, c, M, ld, twc, tid); break;
    case 4: cross_otf<4>(slot, c, M, ld, twc, tid); break;
    case 6: cross_otf<6>(slot, c, M, ld, twc, tid); break;
    case 8: cross_otf<8>(slot, c, M, ld, twc, tid); break;
    case 9: cross_otf<9>(slot, c, M, ld, twc, tid); break;
    case 12: cross_otf<12>(slot, c, M, ld, twc, tid); break;
    default: cross_otf<16>(slot, c, M, ld, twc, tid); break;
  }
}

// Local FFT by the runtime plan (local sizes outside the compile-time menu).
__device__ __noinline__ void bp_local_runtime(float2* s, const FftGeom* g, const float2* row, const float2* twl) {
  first_pass_dispatch<16>(s, *g, ExchangeLoader{row}, threadIdx.x, kBpThreads);
  local_passes<16>(s, *g, 1, twl, threadIdx.x, kBpThreads);
}

// ---- top-K --------------------------------------------------------------------
// Bins of a beam in row layout, written by the previous launch: bin q*CC + r
// is element q of row r (rows M apart).
struct RowBins {
  const float2* rows;
  uint32_t M;
  SPX_DEV float2 operator()(uint32_t r, uint32_t q) const { return __ldg(rows + (size_t)r * M + q); }
};

// The strict local maxima of bins [start, end) of one beam, folded into the
// warp's sorted top-K list (lane l holds entry l; keys |X| bits, then ~bin).
// A lane owns column q: bins q*CC + r (r < CC), one load per row, so a warp
// reads 32 consecutive columns of each row with CC loads in flight.  Each |X|
// is computed once; the neighbours across a column edge come from the next
// lane (or a load at the warp's edge).  The lists depend only on the set of
// candidates, not on the order they are visited in.
template <uint32_t CC, uint32_t NT, typename Bins>
SPX_DEV uint64_t bt_scan(const Bins& bins, uint32_t start, uint32_t end, uint32_t K, uint32_t lane,
                         uint32_t warp) {
  auto bin = [&](uint32_t k) { return bins(k % CC, k / CC); };
  uint64_t mine = 0;
  const uint32_t q_lo = (start - 1) / CC, q_hi = end / CC;
  for (uint32_t q0 = q_lo + warp * 32; q0 <= q_hi; q0 += NT) {
    const uint32_t q = q0 + lane;
    float2 z[CC];
#pragma unroll
    for (uint32_t r = 0; r < CC; ++r) {
      const uint32_t k = q * CC + r;
      z[r] = make_float2(0.f, 0.f);
      if (q <= q_hi && k + 1 >= start && k <= end) z[r] = bins(r, q);
    }
    float m[CC];
#pragma unroll
    for (uint32_t r = 0; r < CC; ++r) m[r] = mag_rn(z[r]);
    float left = __shfl_up_sync(0xffffffffu, m[CC - 1], 1);  // bin q*CC - 1
    float right = __shfl_down_sync(0xffffffffu, m[0], 1);    // bin (q + 1)*CC
    if (lane == 0 && q * CC >= start && q * CC < end) left = mag_rn(bin(q * CC - 1));
    if (lane == 31 && q * CC + CC - 1 >= start && q * CC + CC - 1 < end) right = mag_rn(bin(q * CC + CC));
#pragma unroll
    for (uint32_t r = 0; r < CC; ++r) {
      const uint32_t k = q * CC + r;
      const float c = m[r];
      const float lft = r == 0 ? left : m[r == 0 ? 0 : r - 1];
      const float rgt = r + 1 == CC ? right : m[r + 1 < CC ? r + 1 : r];
      const bool cand = q <= q_hi && k >= start && k < end && c > lft && c > rgt;
      const uint64_t key = ((uint64_t)__float_as_uint(c) << 32) | (uint32_t)(~k);
      const uint64_t kth = __shfl_sync(0xffffffffu, mine, K - 1);
      uint32_t want = __ballot_sync(0xffffffffu, cand && key > kth);
      while (want) {
        const int src = __ffs(want) - 1;
        want &= want - 1;
        mine = warp_list_insert(mine, __shfl_sync(0xffffffffu, key, src), lane);
      }
    }
  }
  return mine;
}

// The K largest strict local maxima of every beam's spectrum (one CTA per
// beam; beam_list orders the CTAs, largest spectra first): per-warp lists
// merged by warp 0, which writes the MaxValues with the rules and arithmetic
// of topk_kernel (|X| descending, ties by lower bin, parabolic refinement on
// the |X| of the neighbours).
// Six CTAs per SM (42 registers, 48 bytes spilled): more loads of the
// beams' rows in flight than at four (no spill); uneven step 0.759 -> 0.744 ms.
__global__ void __launch_bounds__(kBtThreads, 6)
topk_batch_kernel(const float2* __restrict__ xch, const BatchBeam* __restrict__ beams,
                  const BatchGeom* __restrict__ geoms, const uint32_t* __restrict__ beam_list, TopkArgs a) {
  __shared__ uint64_t lists[kBtThreads / 32][32];
  const uint32_t beam = beam_list[blockIdx.x];
  const BatchBeam bm = beams[beam];
  const uint32_t nfft = bm.nfft;
  uint32_t start = a.start == 0 ? 1 : a.start, end = a.end == 0 ? nfft / 2 : a.end;
  if (end >= nfft) end = nfft - 1;
  const uint32_t C = geoms[bm.geom].g.C, M = geoms[bm.geom].g.M;
  const RowBins bins{xch + bm.spec_off, M};
  const uint32_t cmagic = 0xFFFFFFFFu / C + 1u;  // k div C = umulhi(k, cmagic) (k * C < 2^32)
  auto bin = [&](uint32_t k) -> float2 {
    const uint32_t q = C == 1 ? k : __umulhi(k, cmagic);
    return bins(k - q * C, q);
  };
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint64_t mine = 0;
  if (start < end) {
    switch (C) {  // the same for the whole CTA
      case 1: mine = bt_scan<1, kBtThreads>(bins, start, end, a.K, lane, warp); break;
      case 2: mine = bt_scan<2, kBtThreads>(bins, start, end, a.K, lane, warp); break;
      case 3: mine = bt_scan<3, kBtThreads>(bins, start, end, a.K, lane, warp); break;
      case 4: mine = bt_scan<4, kBtThreads>(bins, start, end, a.K, lane, warp); break;
      case 6: mine = bt_scan<6, kBtThreads>(bins, start, end, a.K, lane, warp); break;
      case 8: mine = bt_scan<8, kBtThreads>(bins, start, end, a.K, lane, warp); break;
      case 9: mine = bt_scan<9, kBtThreads>(bins, start, end, a.K, lane, warp); break;
      case 12: mine = bt_scan<12, kBtThreads>(bins, start, end, a.K, lane, warp); break;
      default: mine = bt_scan<16, kBtThreads>(bins, start, end, a.K, lane, warp); break;
    }
  }
  mine = merge_warp_lists(&lists[0][0], mine, kBtThreads / 32, a.K, warp, lane);
  if (warp != 0) return;
  const uint32_t n = __popc(__ballot_sync(0xffffffffu, lane < a.K && mine != 0));
  if (lane == 0) a.counts[beam] = n;
  if (lane < n) {
    const uint32_t k = ~(uint32_t)mine;
    const float bw = __fdiv_rn(a.fs, (float)nfft);
    const float yc = __uint_as_float((uint32_t)(mine >> 32));
    const float yl = mag_rn(bin(k - 1)), yr = mag_rn(bin(k + 1));
    float fo = 0.f, rf = __fmul_rn((float)k, bw);
    if (a.refine == SPX_REFINE_PARABOLIC) {
      const float denom = __fadd_rn(__fsub_rn(yl, __fmul_rn(2.0f, yc)), yr);
      if (fabsf(denom) > 1e-10f) {
        float q = __fdiv_rn(__fmul_rn(0.5f, __fsub_rn(yl, yr)), denom);
        q = fminf(fmaxf(q, -0.5f), 0.5f);
        fo = q;
        rf = __fmul_rn(__fadd_rn((float)k, fo), bw);
      }
    }
    const float2 z = bin(k);
    a.out[(size_t)beam * a.K + lane] =
        MaxValueDev{k, z.x, z.y, yc, __fmul_rn(atan2f(z.y, z.x), kRadToDeg), fo, rf, 0u};
  }
}

__global__ void __launch_bounds__(kBpThreads, 1) fft_batch_kernel(BatchArgs a) {
  extern __shared__ float2 s[];
  cg::cluster_group cl = cg::this_cluster();
  // L2 prefetch of the samples the CTA one residency wave later reads first
  if (a.ahead && blockIdx.x + a.ahead < gridDim.x) {
    const BatchCta f = a.ctas[blockIdx.x + a.ahead];
    if (f.beam != kIdle) {
      const BatchBeam* fb = a.beams + f.beam;
      const FftGeom* fg = &a.geoms[fb->geom].g;
      prefetch_beam_part(a.in + fb->in_off, fb->n_point, fg->C, fg->M, f.c, threadIdx.x, kBpThreads);
    }
  }
  const BatchCta d = a.ctas[blockIdx.x];
  const bool active = d.beam != kIdle;
  if (active) {
    const BatchBeam* bm = a.beams + d.beam;
    const BatchGeom* bg = a.geoms + bm->geom;
    bp_prepare(&bg->g, a.xch + bm->spec_off, d.c, a.in + bm->in_off, bm->n_point, a.window, bg->twc);
  }
  cl.sync();  // every CTA of the cluster exactly once: the beams' cross stages are in their slots
  if (!active) return;
  const BatchBeam* bm = a.beams + d.beam;
  const BatchGeom* bg = a.geoms + bm->geom;
  float2* row = a.xch + bm->spec_off + (size_t)d.c * bg->g.M;
  // row c was read by this CTA alone: it takes the CTA's spectrum row
  if (bg->g.ept != 16 ||
      !ct_menu_fft<(int)kBpThreads>(bg->g.M, s, ExchangeLoader{row}, bg->twl, threadIdx.x, RowOut{row})) {
    bp_local_runtime(s, &bg->g, row, bg->twl);
    for (uint32_t i = threadIdx.x; i < bg->g.M; i += kBpThreads) __stcg(row + i, s[sw(i)]);
  }
}

}  // namespace spx

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
using namespace spx;

struct LaunchSet {  // one FFT launch (packed CTA table, cluster size) and its top-K launch
  uint32_t nfft = 0;  // 0: every beam of the batch, else the beams of this nfft
  BatchCta* d_ctas = nullptr;
  uint32_t* d_beam_list = nullptr;  // the top-K launch's beams, largest spectra first
  uint32_t n_ctas = 0, cluster = 1, beams = 0;
};

struct spx_batch {
  int device = 0;
  uint32_t beams = 0, window = 0, K = 8, start = 0, end = 0, refine = 1;
  float fs = 1.0f;
  std::vector<uint32_t> n_point, nfft;
  std::map<uint32_t, uint32_t> local;  // nfft -> local FFT size M of its plan (C = nfft / M)
  uint32_t cluster_pref = 0;           // CTAs per cluster of the single launch (0: the largest C)
  uint64_t in_total = 0, spec_total = 0;
  LaunchSet all;                       // the single batched launch
  std::vector<LaunchSet> per_size;     // one launch per distinct nfft
  BatchBeam* d_beams = nullptr;
  BatchGeom* d_geoms = nullptr;
  float2* d_xch = nullptr;
  cudaGraphExec_t graph = nullptr;
  std::vector<void*> tables;           // freed on rebuild
  ~spx_batch() {
    if (graph) cudaGraphExecDestroy(graph);
    for (void* p : tables) cudaFree(p);
    if (d_xch) cudaFree(d_xch);
  }
};

namespace {

constexpr uint32_t kClusterSizes[] = {1, 2, 3, 4, 6, 8, 9, 12, 16};

template <typename T>
spx_status upload(spx_ctx* ctx, spx_batch* b, const std::vector<T>& v, T** out) {
  *out = nullptr;
  if (v.empty()) return SPX_OK;
  cudaError_t e = cudaMalloc(out, v.size() * sizeof(T));
  if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaMalloc(batch tables)");
  b->tables.push_back(*out);
  e = cudaMemcpy(*out, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaMemcpy(batch tables)");
  return SPX_OK;
}

// Local sizes a batch may run nfft with: M = nfft / C for the cluster sizes
// C a batch takes, M <= 16384, a geometry the plan builder produces.
std::vector<uint32_t> local_candidates(uint32_t nfft) {
  std::vector<uint32_t> v;
  for (uint32_t c : kClusterSizes) {
    if (nfft % c || nfft / c > kMaxLocal || nfft / c < 2) continue;
    FftGeom g{};
    if (build_geom(nfft, &g, 16, c == 1 ? (uint32_t)kPrefLocalCluster : std::max<uint32_t>(1024u, nfft / c)) &&
        g.M == nfft / c)
      v.push_back(nfft / c);
  }
  return v;
}

// The context's plan of nfft with local size M (16 points per thread): it
// becomes the plan of every call on the context for nfft.
spx_status plan_with_local(spx_ctx* ctx, uint32_t nfft, uint32_t M, const FftPlan** plan) {
  ctx->tuning[nfft] = {16u, M == nfft ? (uint32_t)kPrefLocalCluster : std::max<uint32_t>(1024u, M)};
  spx_status st = get_plan(ctx, nfft, plan);
  if (st != SPX_OK) return st;
  if ((*plan)->big || (*plan)->g.C > kBtMaxC || (*plan)->g.M != M)
    return fail(ctx, SPX_ERR_UNSUPPORTED, "batch: nfft " + std::to_string(nfft) + " with local size " +
                                              std::to_string(M));
  return SPX_OK;
}

// Packs the given beams into clusters of `cl` CTAs: beams by cluster size,
// then transform size, largest first, each into the first cluster with room
// (first-fit decreasing); the CTA table in cluster order, idle CTAs filling
// the clusters' unused ranks.
std::vector<BatchCta> pack(std::vector<uint32_t> ids, const std::vector<uint32_t>& group,
                           const std::vector<uint32_t>& nfft, uint32_t cl) {
  std::stable_sort(ids.begin(), ids.end(), [&](uint32_t a, uint32_t b) {
    return group[a] != group[b] ? group[a] > group[b] : nfft[a] > nfft[b];
  });
  std::vector<std::vector<uint32_t>> clusters;  // beams per cluster
  std::vector<uint32_t> used;
  for (uint32_t beam : ids) {
    size_t j = 0;
    while (j < clusters.size() && used[j] + group[beam] > cl) ++j;
    if (j == clusters.size()) {
      clusters.emplace_back();
      used.push_back(0);
    }
    clusters[j].push_back(beam);
    used[j] += group[beam];
  }
  std::vector<BatchCta> ctas;
  ctas.reserve(clusters.size() * cl);
  for (const auto& cb : clusters) {
    uint32_t r = 0;
    for (uint32_t beam : cb)
      for (uint32_t c = 0; c < group[beam]; ++c, ++r) ctas.push_back(BatchCta{beam, c});
    for (; r < cl; ++r) ctas.push_back(BatchCta{kIdle, 0});
  }
  return ctas;
}

// The most CTAs any beam of the batch takes (C = nfft / M of its plan).
uint32_t largest_c(const spx_batch* b) {
  uint32_t c = 1;
  for (const auto& kv : b->local) c = std::max(c, kv.first / kv.second);
  return c;
}

// Tables and launch sets from the batch's plan choices.
spx_status build(spx_ctx* ctx, spx_batch* b) {
  for (void* p : b->tables) cudaFree(p);
  b->tables.clear();
  b->d_beams = nullptr;
  b->d_geoms = nullptr;
  std::map<uint32_t, uint32_t> geom_of;  // nfft -> geometry index
  std::vector<BatchGeom> geoms;
  for (auto& kv : b->local) {
    const FftPlan* plan = nullptr;
    spx_status st = plan_with_local(ctx, kv.first, kv.second, &plan);
    if (st != SPX_OK) return st;
    geom_of[kv.first] = (uint32_t)geoms.size();
    geoms.push_back(BatchGeom{plan->g, plan->d_tw_local, plan->d_tw_cross});
  }
  std::vector<BatchBeam> beams(b->beams);
  std::vector<uint32_t> group(b->beams);
  uint64_t in_off = 0, spec_off = 0;
  for (uint32_t i = 0; i < b->beams; ++i) {
    beams[i] = BatchBeam{in_off, spec_off, b->n_point[i], b->nfft[i], geom_of[b->nfft[i]], 0};
    group[i] = geoms[geom_of[b->nfft[i]]].g.C;
    in_off += b->n_point[i];
    spec_off += (b->nfft[i] + 31u) & ~31u;  // 256-byte aligned spectra
  }
  b->in_total = in_off;
  b->spec_total = spec_off;
  spx_status st = upload(ctx, b, beams, &b->d_beams);
  if (st == SPX_OK) st = upload(ctx, b, geoms, &b->d_geoms);
  if (st != SPX_OK) return st;
  auto make_set = [&](const std::vector<uint32_t>& ids, uint32_t nfft, LaunchSet* ls) -> spx_status {
    uint32_t cl = 1;
    for (uint32_t id : ids) cl = std::max(cl, group[id]);
    // the single launch may use larger clusters than its largest beam needs
    // (several beams per cluster): how many fit at once depends on how the
    // cluster size divides the GPU's SM groups
    if (nfft == 0 && b->cluster_pref > cl) cl = b->cluster_pref;
    const std::vector<BatchCta> ctas = pack(ids, group, b->nfft, cl);
    ls->nfft = nfft;
    ls->n_ctas = (uint32_t)ctas.size();
    ls->cluster = cl;
    ls->beams = (uint32_t)ids.size();
    std::vector<uint32_t> by_size(ids);
    std::stable_sort(by_size.begin(), by_size.end(),
                     [&](uint32_t x, uint32_t y) { return b->nfft[x] > b->nfft[y]; });
    spx_status s2 = upload(ctx, b, ctas, &ls->d_ctas);
    if (s2 == SPX_OK) s2 = upload(ctx, b, by_size, &ls->d_beam_list);
    return s2;
  };
  std::vector<uint32_t> all(b->beams);
  for (uint32_t i = 0; i < b->beams; ++i) all[i] = i;
  st = make_set(all, 0, &b->all);
  if (st != SPX_OK) return st;
  std::map<uint32_t, std::vector<uint32_t>, std::greater<uint32_t>> by_size;
  for (uint32_t i = 0; i < b->beams; ++i) by_size[b->nfft[i]].push_back(i);
  b->per_size.clear();
  for (auto& kv : by_size) {
    b->per_size.emplace_back();
    st = make_set(kv.second, kv.first, &b->per_size.back());
    if (st != SPX_OK) return st;
  }
  if (b->graph) {  // recorded with the old tables
    cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
  }
  return SPX_OK;
}

// The FFT launch and the top-K launch of a launch set.
spx_status launch_set(spx_ctx* ctx, spx_batch* b, const LaunchSet& ls, const void* d_in,
                      spx_max_value* d_out, uint32_t* d_counts) {
  const void* kfn = (const void*)fft_batch_kernel;
  cudaError_t e = configure_kernel(kfn, kBpSmem);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "configure fft_batch_kernel");
  BatchArgs a{};
  a.in = static_cast<const float2*>(d_in);
  a.beams = b->d_beams;
  a.geoms = b->d_geoms;
  a.ctas = ls.d_ctas;
  a.window = b->window;
  a.ahead = ctx->input_on_host ? 0u : resident_ctas(kfn, kBpThreads, kBpSmem, ls.cluster);
  a.xch = b->d_xch;
  void* args[] = {(void*)&a};
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(ls.n_ctas, 1, 1);
  cfg.blockDim = dim3(kBpThreads, 1, 1);
  cfg.dynamicSmemBytes = kBpSmem;
  cfg.stream = ctx->stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = ls.cluster;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  e = cudaLaunchKernelExC(&cfg, kfn, args);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "launch fft_batch_kernel");
  const TopkArgs tk{reinterpret_cast<MaxValueDev*>(d_out), d_counts, b->K, b->start, b->end, b->refine, b->fs};
  topk_batch_kernel<<<ls.beams, kBtThreads, 0, ctx->stream>>>(b->d_xch, b->d_beams, b->d_geoms, ls.d_beam_list, tk);
  e = cudaGetLastError();
  return e == cudaSuccess ? SPX_OK : cuda_fail(ctx, e, "launch topk_batch_kernel");
}

struct Guard {
  int prev = -1;
  explicit Guard(int dev) {
    if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
    if (prev != dev) cudaSetDevice(dev);
  }
  ~Guard() {
    int cur = -1;
    if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
  }
};

spx_status check_run_args(spx_ctx* ctx, spx_batch* batch, const void* d_in, const void* d_out,
                          const void* d_counts, const char* what) {
  if (!d_in || !d_out || !d_counts) return fail(ctx, SPX_ERR_INVALID_ARG, std::string(what) + ": null pointer");
  if (batch->device != ctx->device)
    return fail(ctx, SPX_ERR_INVALID_ARG, std::string(what) + ": the batch belongs to another device");
  return SPX_OK;
}

std::string device_arch(int device) {
  cudaDeviceProp prop{};
  if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return "";
  return "sm_" + std::to_string(prop.major) + std::to_string(prop.minor);
}

}  // namespace

extern "C" {

spx_status spx_batch_create(spx_ctx* ctx, uint32_t beams, const uint32_t* n_points,
                            const uint32_t* nffts, uint32_t window,
                            const spx_peak_params* params, spx_batch** out) {
  if (!ctx || !out) return SPX_ERR_INVALID_ARG;
  *out = nullptr;
  if (!params || !n_points) return fail(ctx, SPX_ERR_INVALID_ARG, "spx_batch_create: null argument");
  if (beams == 0) return fail(ctx, SPX_ERR_INVALID_ARG, "spx_batch_create: beams must be > 0");
  if (params->mode != SPX_PEAK_TOPK)
    return fail(ctx, SPX_ERR_UNSUPPORTED, "spx_batch_create: only SPX_PEAK_TOPK batches are built");
  if (params->max_per_beam < 1 || params->max_per_beam > 32)
    return fail(ctx, SPX_ERR_INVALID_ARG, "spx_batch_create: K must be in [1, 32]");
  if (params->thresh_sigma != 0.0f)
    return fail(ctx, SPX_ERR_UNSUPPORTED, "spx_batch_create: thresh_sigma must be 0");
  if (params->refine > SPX_REFINE_PARABOLIC || window > SPX_WINDOW_BLACKMAN_HARRIS)
    return fail(ctx, SPX_ERR_INVALID_ARG, "spx_batch_create: bad refine or window");
  Guard gd(ctx->device);
  auto* b = new (std::nothrow) spx_batch();
  if (!b) return SPX_ERR_OUT_OF_MEMORY;
  b->device = ctx->device;
  b->beams = beams;
  b->window = window;
  b->K = params->max_per_beam;
  b->start = params->search_start;
  b->end = params->search_end;
  b->refine = params->refine;
  b->fs = params->sample_rate;
  b->n_point.assign(n_points, n_points + beams);
  b->nfft.resize(beams);
  for (uint32_t i = 0; i < beams; ++i) {
    const uint32_t n = nffts && nffts[i] ? nffts[i] : spx_next_smooth23(n_points[i]);
    if (n_points[i] == 0 || n < n_points[i] || n < 3 || !spx_fft_size_supported(n)) {
      delete b;
      return fail(ctx, SPX_ERR_INVALID_ARG,
                  "spx_batch_create: beam " + std::to_string(i) + " has an unsupported size");
    }
    if (big_size(n) || huge_size(n)) {  // multi-launch transforms: not slots of the batch kernel
      delete b;
      return fail(ctx, SPX_ERR_UNSUPPORTED,
                  "spx_batch_create: beam " + std::to_string(i) + " needs nfft " + std::to_string(n) +
                      "; transforms of 2^19 points and more run through spx_fft_peaks, not in a batch");
    }
    b->nfft[i] = n;
    if (!b->local.count(n)) {
      // the context's plan for n (a size set by spx_set_fft_tuning or an
      // earlier autotune, 16 points per thread), else the default one
      FftGeom g{};
      auto te = ctx->tuning.find(n);
      const uint32_t pref = te != ctx->tuning.end() ? te->second.second : (uint32_t)kPrefLocalCluster;
      if (!build_geom(n, &g, 16, pref) && !build_geom(n, &g, 16, kPrefLocalCluster)) {
        delete b;
        return fail(ctx, SPX_ERR_INVALID_ARG, "spx_batch_create: nfft " + std::to_string(n) + " has no plan");
      }
      b->local[n] = g.M;
    }
  }
  spx_status st = build(ctx, b);
  if (st == SPX_OK) {
    cudaError_t e = cudaMalloc(&b->d_xch, b->spec_total * sizeof(float2));
    if (e != cudaSuccess) st = cuda_fail(ctx, e, "cudaMalloc(batch exchange slots)");
  }
  if (st != SPX_OK) {
    delete b;
    return st;
  }
  *out = b;
  return SPX_OK;
}

spx_status spx_batch_destroy(spx_batch* batch) {
  if (!batch) return SPX_OK;
  Guard gd(batch->device);
  delete batch;
  return SPX_OK;
}

uint64_t spx_batch_input_samples(const spx_batch* batch) { return batch ? batch->in_total : 0; }

spx_status spx_batch_run(spx_ctx* ctx, spx_batch* batch, const void* d_in, spx_max_value* d_out,
                         uint32_t* d_counts) {
  if (!ctx || !batch) return SPX_ERR_INVALID_ARG;
  spx_status st = check_run_args(ctx, batch, d_in, d_out, d_counts, "spx_batch_run");
  if (st != SPX_OK) return st;
  Guard gd(ctx->device);
  return launch_set(ctx, batch, batch->all, d_in, d_out, d_counts);
}

spx_status spx_batch_run_per_size(spx_ctx* ctx, spx_batch* batch, const void* d_in,
                                  spx_max_value* d_out, uint32_t* d_counts) {
  if (!ctx || !batch) return SPX_ERR_INVALID_ARG;
  spx_status st = check_run_args(ctx, batch, d_in, d_out, d_counts, "spx_batch_run_per_size");
  if (st != SPX_OK) return st;
  Guard gd(ctx->device);
  for (const LaunchSet& ls : batch->per_size) {
    st = launch_set(ctx, batch, ls, d_in, d_out, d_counts);
    if (st != SPX_OK) return st;
  }
  return SPX_OK;
}

spx_status spx_batch_capture(spx_ctx* ctx, spx_batch* batch, const void* d_in,
                             spx_max_value* d_out, uint32_t* d_counts) {
  if (!ctx || !batch) return SPX_ERR_INVALID_ARG;
  spx_status st = check_run_args(ctx, batch, d_in, d_out, d_counts, "spx_batch_capture");
  if (st != SPX_OK) return st;
  if (!ctx->stream)
    return fail(ctx, SPX_ERR_INVALID_ARG, "spx_batch_capture: set a non-default stream first");
  Guard gd(ctx->device);
  // resolve lazy set-up (attributes, occupancy) before capturing
  cudaError_t e = configure_kernel((const void*)fft_batch_kernel, kBpSmem);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "configure fft_batch_kernel");
  resident_ctas((const void*)fft_batch_kernel, kBpThreads, kBpSmem, batch->all.cluster);
  e = cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaStreamBeginCapture");
  st = launch_set(ctx, batch, batch->all, d_in, d_out, d_counts);
  cudaGraph_t graph = nullptr;
  e = cudaStreamEndCapture(ctx->stream, &graph);
  if (st != SPX_OK) {
    if (graph) cudaGraphDestroy(graph);
    return st;
  }
  if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaStreamEndCapture");
  if (batch->graph) cudaGraphExecDestroy(batch->graph);
  batch->graph = nullptr;
  e = cudaGraphInstantiate(&batch->graph, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaGraphInstantiate");
  return SPX_OK;
}

spx_status spx_batch_replay(spx_ctx* ctx, spx_batch* batch) {
  if (!ctx || !batch) return SPX_ERR_INVALID_ARG;
  if (!batch->graph) return fail(ctx, SPX_ERR_INVALID_ARG, "spx_batch_replay: no captured graph");
  Guard gd(ctx->device);
  cudaError_t e = cudaGraphLaunch(batch->graph, ctx->stream);
  return e == cudaSuccess ? SPX_OK : cuda_fail(ctx, e, "cudaGraphLaunch");
}

spx_status spx_batch_tune(spx_ctx* ctx, spx_batch* batch, uint32_t points_per_thread,
                          uint32_t points_per_cta) {
  if (!ctx || !batch) return SPX_ERR_INVALID_ARG;
  if (points_per_thread != 16)
    return fail(ctx, SPX_ERR_UNSUPPORTED,
                "spx_batch_tune: batches run 16 points per thread (1024-thread CTAs of up to 16384 points)");
  if (points_per_cta == 0) points_per_cta = kPrefLocalCluster;
  if (points_per_cta < 1024 || points_per_cta > kMaxLocal)
    return fail(ctx, SPX_ERR_INVALID_ARG, "spx_batch_tune: points_per_cta out of range");
  Guard gd(ctx->device);
  for (auto& kv : batch->local) {
    FftGeom g{};
    if (build_geom(kv.first, &g, 16, points_per_cta) && g.C <= kBtMaxC) kv.second = g.M;
  }
  return build(ctx, batch);
}

uint32_t spx_batch_local_size(const spx_batch* batch, uint32_t nfft) {
  if (!batch) return 0;
  auto it = batch->local.find(nfft);
  return it == batch->local.end() ? 0u : it->second;
}

spx_status spx_batch_set_local_size(spx_ctx* ctx, spx_batch* batch, uint32_t nfft, uint32_t local_size) {
  if (!ctx || !batch) return SPX_ERR_INVALID_ARG;
  auto it = batch->local.find(nfft);
  if (it == batch->local.end())
    return fail(ctx, SPX_ERR_INVALID_ARG, "spx_batch_set_local_size: no beam of the batch has nfft " +
                                              std::to_string(nfft));
  const std::vector<uint32_t> cand = local_candidates(nfft);
  if (std::find(cand.begin(), cand.end(), local_size) == cand.end())
    return fail(ctx, SPX_ERR_INVALID_ARG, "spx_batch_set_local_size: " + std::to_string(local_size) +
                                              " is not a local size of nfft " + std::to_string(nfft));
  Guard gd(ctx->device);
  it->second = local_size;
  return build(ctx, batch);
}

spx_status spx_batch_autotune(spx_ctx* ctx, spx_batch* batch, const void* d_in,
                              spx_max_value* d_out, uint32_t* d_counts, uint32_t* sizes_tuned,
                              uint32_t* sizes_changed) {
  if (!ctx || !batch) return SPX_ERR_INVALID_ARG;
  spx_status st = check_run_args(ctx, batch, d_in, d_out, d_counts, "spx_batch_autotune");
  if (st != SPX_OK) return st;
  Guard gd(ctx->device);
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
    if (e0) cudaEventDestroy(e0);
    return fail(ctx, SPX_ERR_CUDA, "spx_batch_autotune: cudaEventCreate");
  }
  uint32_t tuned = 0, changed = 0;
  std::vector<uint32_t> sizes;
  for (const LaunchSet& ls : batch->per_size) sizes.push_back(ls.nfft);
  // per distinct nfft, largest first: the whole batch timed with each
  // candidate local size for that nfft (the others as chosen so far); the
  // current plan stays unless another is faster by more than 2 %.  The whole
  // batch, not the size alone, because the sizes share one launch: a size's
  // cluster size, for one, is every cluster's.
  auto time_batch = [&](float* ms) -> spx_status {
    spx_status s2 = SPX_OK;
    for (int w = 0; w < 2 && s2 == SPX_OK; ++w) s2 = launch_set(ctx, batch, batch->all, d_in, d_out, d_counts);
    cudaEventRecord(e0, ctx->stream);
    for (int rep = 0; rep < 5 && s2 == SPX_OK; ++rep) s2 = launch_set(ctx, batch, batch->all, d_in, d_out, d_counts);
    cudaEventRecord(e1, ctx->stream);
    if (s2 != SPX_OK) return s2;
    if (cudaEventSynchronize(e1) != cudaSuccess) return fail(ctx, SPX_ERR_CUDA, "spx_batch_autotune: cudaEventSynchronize");
    cudaEventElapsedTime(ms, e0, e1);
    return SPX_OK;
  };
  for (uint32_t n : sizes) {
    const std::vector<uint32_t> cand = local_candidates(n);
    if (cand.size() < 2) continue;
    const uint32_t was = batch->local[n];
    uint32_t best_m = was;
    float best = 1e30f, best_was = 1e30f;
    for (uint32_t m : cand) {
      batch->local[n] = m;
      st = build(ctx, batch);
      if (st != SPX_OK) break;
      float ms = 0.f;
      st = time_batch(&ms);
      if (st != SPX_OK) break;
      if (m == was) best_was = ms;
      if (ms < best) {
        best = ms;
        best_m = m;
      }
    }
    if (best_m != was && best_was < 1e30f && best > 0.98f * best_was) best_m = was;
    batch->local[n] = best_m;
    if (st != SPX_OK) break;
    ++tuned;
    if (best_m != was) ++changed;
  }
  // then the cluster size of the single launch: from the largest C to 16
  if (st == SPX_OK) {
    const uint32_t maxc = largest_c(batch);
    const uint32_t was = batch->cluster_pref;
    uint32_t best_cl = was;
    float best = 1e30f, best_was = 1e30f;
    for (uint32_t cl = maxc; cl <= kBtMaxC && st == SPX_OK; ++cl) {
      batch->cluster_pref = cl == maxc ? 0u : cl;
      if (resident_ctas((const void*)fft_batch_kernel, kBpThreads, kBpSmem, cl) == 0) continue;
      st = build(ctx, batch);
      float ms = 0.f;
      if (st == SPX_OK) st = time_batch(&ms);
      if (st != SPX_OK) break;
      if (batch->cluster_pref == was) best_was = ms;
      if (ms < best) {
        best = ms;
        best_cl = batch->cluster_pref;
      }
    }
    if (best_cl != was && best_was < 1e30f && best > 0.98f * best_was) best_cl = was;
    batch->cluster_pref = best_cl;
    if (best_cl != was) ++changed;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  spx_status st2 = build(ctx, batch);
  if (st == SPX_OK) st = st2;
  if (sizes_tuned) *sizes_tuned = tuned;
  if (sizes_changed) *sizes_changed = changed;
  return st;
}

// Plan cache: one JSON object per file,
//   {"arch": "sm_103", "plans": {"<nfft>": <local size>, ...}, "cluster": <CTAs per cluster, 0: the largest C>}
spx_status spx_batch_save_plans(spx_ctx* ctx, const spx_batch* batch, const char* path) {
  if (!ctx || !batch) return SPX_ERR_INVALID_ARG;
  if (!path) return fail(ctx, SPX_ERR_INVALID_ARG, "spx_batch_save_plans: path is null");
  const std::string arch = device_arch(batch->device);
  if (arch.empty()) return fail(ctx, SPX_ERR_CUDA, "spx_batch_save_plans: cudaGetDeviceProperties");
  std::ofstream f(path);
  if (!f) return fail(ctx, SPX_ERR_INVALID_ARG, std::string("spx_batch_save_plans: cannot write ") + path);
  f << "{\"arch\": \"" << arch << "\", \"plans\": {";
  bool first = true;
  for (const auto& kv : batch->local) {
    f << (first ? "" : ", ") << "\"" << kv.first << "\": " << kv.second;
    first = false;
  }
  f << "}, \"cluster\": " << batch->cluster_pref << "}\n";
  f.close();
  return f ? SPX_OK : fail(ctx, SPX_ERR_INVALID_ARG, "spx_batch_save_plans: write failed");
}

spx_status spx_batch_load_plans(spx_ctx* ctx, spx_batch* batch, const char* path, uint32_t* applied) {
  if (!ctx || !batch) return SPX_ERR_INVALID_ARG;
  if (applied) *applied = 0;
  if (!path) return fail(ctx, SPX_ERR_INVALID_ARG, "spx_batch_load_plans: path is null");
  std::ifstream f(path);
  if (!f) return fail(ctx, SPX_ERR_INVALID_ARG, std::string("spx_batch_load_plans: cannot read ") + path);
  std::stringstream ss;
  ss << f.rdbuf();
  const std::string text = ss.str();
  const std::string arch = device_arch(batch->device);
  if (arch.empty() || text.find("\"arch\": \"" + arch + "\"") == std::string::npos)
    return fail(ctx, SPX_ERR_INVALID_ARG, "spx_batch_load_plans: the file holds no plans for " + arch);
  const size_t p0 = text.find("\"plans\"");
  const size_t open = p0 == std::string::npos ? std::string::npos : text.find('{', p0);
  const size_t close = open == std::string::npos ? std::string::npos : text.find('}', open);
  if (close == std::string::npos)
    return fail(ctx, SPX_ERR_INVALID_ARG, "spx_batch_load_plans: no \"plans\" object");
  uint32_t n_applied = 0;
  size_t p = open + 1;
  while (p < close) {  // "nfft": M pairs
    const size_t q1 = text.find('"', p);
    if (q1 == std::string::npos || q1 > close) break;
    const size_t q2 = text.find('"', q1 + 1);
    const size_t colon = text.find(':', q2);
    if (q2 == std::string::npos || colon == std::string::npos || colon > close) break;
    const unsigned long nfft = std::strtoul(text.c_str() + q1 + 1, nullptr, 10);
    const unsigned long m = std::strtoul(text.c_str() + colon + 1, nullptr, 10);
    auto it = batch->local.find((uint32_t)nfft);
    if (it != batch->local.end()) {
      const std::vector<uint32_t> cand = local_candidates((uint32_t)nfft);
      if (std::find(cand.begin(), cand.end(), (uint32_t)m) != cand.end()) {
        it->second = (uint32_t)m;
        ++n_applied;
      }
    }
    const size_t comma = text.find(',', colon);
    p = comma == std::string::npos ? close : comma + 1;
  }
  // "cluster": N (0 = the largest C); applied when valid for the batch
  const size_t pc = text.find("\"cluster\"", close);
  if (pc != std::string::npos) {
    const size_t colon = text.find(':', pc);
    const unsigned long cl = colon == std::string::npos ? 0ul : std::strtoul(text.c_str() + colon + 1, nullptr, 10);
    if (cl <= kBtMaxC && (cl == 0 || cl >= largest_c(batch))) batch->cluster_pref = (uint32_t)cl;
  }
  Guard gd(ctx->device);
  spx_status st = build(ctx, batch);
  if (applied) *applied = n_applied;
  return st;
}

uint32_t spx_batch_cluster(const spx_batch* batch) { return batch ? batch->all.cluster : 0u; }

spx_status spx_batch_set_cluster(spx_ctx* ctx, spx_batch* batch, uint32_t cluster) {
  if (!ctx || !batch) return SPX_ERR_INVALID_ARG;
  if (cluster > kBtMaxC)
    return fail(ctx, SPX_ERR_INVALID_ARG, "spx_batch_set_cluster: at most 16 CTAs per cluster");
  const uint32_t need = largest_c(batch);
  if (cluster != 0 && cluster < need)
    return fail(ctx, SPX_ERR_INVALID_ARG, "spx_batch_set_cluster: a beam of the batch needs " +
                                              std::to_string(need) + " CTAs per cluster");
  Guard gd(ctx->device);
  if (cluster != 0 && resident_ctas((const void*)fft_batch_kernel, kBpThreads, kBpSmem, cluster) == 0)
    return fail(ctx, SPX_ERR_UNSUPPORTED, "spx_batch_set_cluster: no cluster of " + std::to_string(cluster) +
                                              " CTAs fits the device");
  batch->cluster_pref = cluster;
  return build(ctx, batch);
}

}  // extern "C"
