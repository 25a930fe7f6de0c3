// batch.cu — many beams of uneven length and FFT size in one launch.
//
// A batch holds, for B beams with their own n_point and nfft (2^a*3^b), the
// per-size FFT plans, the packing of all beams into clusters of a single
// launch, the device scratch (exchange slots and spectra) and optionally a
// CUDA graph of the whole run.  One run is two launches:
//   1. fft_batch_kernel: every beam's windowed, zero-padded FFT in ONE
//      launch.  The launch has fixed cluster dims Cl (the largest per-beam
//      cluster size); each cluster hosts one or several beams on disjoint
//      rank ranges (first-fit decreasing packing), beams needing no cluster
//      run on single CTAs.  Each CTA leaves its spectrum row in the beam's
//      exchange slot (row c: X[c + C*i] at column i; one row for C = 1):
//      stores in contiguous runs instead of stride-C scatter.
//   2. topk_batch_kernel: the K largest strict local maxima of every beam,
//      one CTA per beam, the same selection rules as spx_topk, reading bin k
//      from row k mod C of the beam's slot.
// The "plain" path runs the same two kernels once per distinct nfft (one
// plan per size, as a per-size library call would), so its results are
// bit-identical to the batched run by construction.
//
// No reference counterpart: DspSpectrum transforms one size per call
// (FFTProcessorROCm, hipfftPlan1d with one nFFT per plan,
// src/fft_func/src/fft_processor_rocm.cpp:152-193).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <map>
#include <vector>

#include "fft_core.cuh"
#include "spx_internal.h"

namespace spx {

constexpr uint32_t kIdle = 0xFFFFFFFFu;

struct BatchBeam {
  uint64_t in_off;    // first sample in the packed input (complex elements)
  uint64_t spec_off;  // first element of the beam's exchange slot (its spectrum rows after the FFT)
  uint32_t n_point, nfft, geom, pad;
};
struct BatchCta {
  uint32_t beam;  // kIdle: this CTA has no work
  uint32_t c;     // rank within the beam's group of CTAs
  uint32_t r0;    // cluster rank of the group's first CTA
  uint32_t pad;
};
struct BatchGeom {
  FftGeom g;
  const float2* twl;
  const float2* twc;
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
                       const float2* twc, uint32_t tid, uint32_t T) {
  const uint32_t S = (M + CR - 1) / CR;
  const uint32_t lo = c * S, hi = min(lo + S, M);
  for (uint32_t n2 = lo + tid; n2 < hi; n2 += T) {
    float2 v[CR];
#pragma unroll
    for (int n1 = 0; n1 < CR; ++n1) v[n1] = ld(n1 * M + n2);
    Dft<CR>::run(v);
    __stcg(slot + n2, v[0]);
#pragma unroll
    for (int k1 = 1; k1 < CR; ++k1)
      __stcg(slot + (size_t)k1 * M + n2, cmul(v[k1], __ldg(twc + (k1 - 1) * M + n2)));
  }
}

template <int EPT>
__global__ void __launch_bounds__(kMaxLocal / EPT, 1)
fft_batch_kernel(const float2* __restrict__ in, const BatchBeam* __restrict__ beams,
                 const BatchCta* __restrict__ ctas, const BatchGeom* __restrict__ geoms,
                 uint32_t window, float2* __restrict__ xch, uint32_t ahead) {
  extern __shared__ float2 s[];
  cg::cluster_group cl = cg::this_cluster();
  const uint32_t tid = threadIdx.x, T = blockDim.x;
  // L2 prefetch for the CTA that starts one residency wave (`ahead` CTAs) later
  if (ahead && blockIdx.x + ahead < gridDim.x) {
    const BatchCta f = ctas[blockIdx.x + ahead];
    if (f.beam != kIdle) {
      const BatchBeam fb = beams[f.beam];
      prefetch_beam_part(in + fb.in_off, fb.n_point, geoms[fb.geom].g.C, geoms[fb.geom].g.M, f.c, tid, T);
    }
  }
  const BatchCta d = ctas[blockIdx.x];
  const bool active = d.beam != kIdle;
  BatchBeam bm{};
  if (active) bm = beams[d.beam];
  // the geometry is read in place from the table (idle CTAs see entry 0 and use none of it)
  const BatchGeom& bg = geoms[active ? bm.geom : 0u];
  const FftGeom& g = bg.g;
  const float2* twl = bg.twl;
  const float2* twc = bg.twc;
  const SampleLoaderOTF ld{in + bm.in_off, bm.n_point, make_window_gen(window, bm.n_point)};
  float2* slot = xch + bm.spec_off;
  if (active && g.C > 1) {
    switch (g.C) {
      case 2: cross_otf<2>(slot, d.c, g.M, ld, twc, tid, T); break;
      case 3: cross_otf<3>(slot, d.c, g.M, ld, twc, tid, T); break;
      case 4: cross_otf<4>(slot, d.c, g.M, ld, twc, tid, T); break;
      case 6: cross_otf<6>(slot, d.c, g.M, ld, twc, tid, T); break;
      case 8: cross_otf<8>(slot, d.c, g.M, ld, twc, tid, T); break;
      case 9: cross_otf<9>(slot, d.c, g.M, ld, twc, tid, T); break;
      case 12: cross_otf<12>(slot, d.c, g.M, ld, twc, tid, T); break;
      default: cross_otf<16>(slot, d.c, g.M, ld, twc, tid, T); break;
    }
  }
  cl.sync();  // every CTA of the cluster exactly once
  if (!active) return;
  float2* row = slot + (size_t)d.c * g.M;  // read by this CTA alone (C > 1)
  if (g.C == 1) {
    first_pass_dispatch<EPT>(s, g, ld, tid, T);
  } else {
    first_pass_dispatch<EPT>(s, g, ExchangeLoader{row}, tid, T);
  }
  local_passes<EPT>(s, g, 1, twl, tid, T);
  for (uint32_t i = tid; i < g.M; i += T) row[i] = s[sw(i)];
}

// Top-K strict local maxima of every beam's spectrum (one CTA per beam),
// the rules of topk_kernel (peak_kernels.cu) on packed, uneven spectra.
constexpr uint32_t kBtThreads = 256;
constexpr uint32_t kBtMaxC = 16;  // CTAs per beam in a batch (cluster size limit)

SPX_DEV uint64_t bt_insert(uint64_t mine, uint64_t x, uint32_t lane) {
  const uint64_t up = __shfl_up_sync(0xffffffffu, mine, 1);
  if (mine >= x) return mine;
  return (lane == 0 || up >= x) ? x : up;
}

// The strict local maxima of bins [start, end) of one beam whose spectrum is
// left in row layout (bin k in row k mod CC, column k div CC; rows M apart),
// folded into the warp's sorted top-K list.  A lane owns column q: bins
// q*CC + r (r < CC), one load per row, so a warp reads 32 consecutive
// columns of each row (256 contiguous bytes) with CC loads in flight.  Each
// |X| is computed once; the neighbours across a column edge come from the
// next lane (or a load at the warp's edge).  The lists depend only on the set
// of candidates, not on the order they are visited in.  The columns cover
// bins start - 1 .. end.
template <uint32_t CC>
SPX_DEV uint64_t bt_scan(const float2* __restrict__ fs_row, uint32_t M, uint32_t start, uint32_t end,
                         uint32_t K, uint32_t lane, uint32_t warp) {
  auto bin = [&](uint32_t k) { return __ldg(fs_row + (size_t)(k % CC) * M + k / CC); };
  uint64_t mine = 0;
  const uint32_t q_lo = (start - 1) / CC, q_hi = end / CC;
  for (uint32_t q0 = q_lo + warp * 32; q0 <= q_hi; q0 += kBtThreads) {
    const uint32_t q = q0 + lane;
    float2 z[CC];
#pragma unroll
    for (uint32_t r = 0; r < CC; ++r) {
      const uint32_t k = q * CC + r;
      z[r] = make_float2(0.f, 0.f);
      if (q <= q_hi && k + 1 >= start && k <= end) z[r] = __ldg(fs_row + (size_t)r * M + q);
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
        mine = bt_insert(mine, __shfl_sync(0xffffffffu, key, src), lane);
      }
    }
  }
  return mine;
}

__global__ void __launch_bounds__(kBtThreads, 4)
topk_batch_kernel(const float2* __restrict__ xch, const BatchBeam* __restrict__ beams,
                  const BatchGeom* __restrict__ geoms, const uint32_t* __restrict__ beam_list, uint32_t K,
                  uint32_t start0, uint32_t end0, float fs, uint32_t refine, MaxValueDev* __restrict__ out,
                  uint32_t* __restrict__ counts) {
  __shared__ uint64_t lists[kBtThreads / 32][32];
  const uint32_t beam = beam_list ? beam_list[blockIdx.x] : blockIdx.x;
  const BatchBeam bm = beams[beam];
  const uint32_t nfft = bm.nfft;
  uint32_t start = start0 == 0 ? 1 : start0, end = end0 == 0 ? nfft / 2 : end0;
  if (end >= nfft) end = nfft - 1;
  // bin k of the beam: row k mod C, column k div C of its slot
  const uint32_t C = geoms[bm.geom].g.C, M = geoms[bm.geom].g.M;
  const uint32_t cmagic = 0xFFFFFFFFu / C + 1u;  // k div C = umulhi(k, cmagic) (k * C < 2^32)
  const float2* fs_row = xch + bm.spec_off;
  auto bin = [&](uint32_t k) -> float2 {
    if (C == 1) return __ldg(fs_row + k);
    const uint32_t q = __umulhi(k, cmagic);
    return __ldg(fs_row + (size_t)(k - q * C) * M + q);
  };
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint64_t mine = 0;
  switch (C) {  // the same for the whole CTA
    case 1: mine = bt_scan<1>(fs_row, M, start, end, K, lane, warp); break;
    case 2: mine = bt_scan<2>(fs_row, M, start, end, K, lane, warp); break;
    case 3: mine = bt_scan<3>(fs_row, M, start, end, K, lane, warp); break;
    case 4: mine = bt_scan<4>(fs_row, M, start, end, K, lane, warp); break;
    case 6: mine = bt_scan<6>(fs_row, M, start, end, K, lane, warp); break;
    case 8: mine = bt_scan<8>(fs_row, M, start, end, K, lane, warp); break;
    case 9: mine = bt_scan<9>(fs_row, M, start, end, K, lane, warp); break;
    case 12: mine = bt_scan<12>(fs_row, M, start, end, K, lane, warp); break;
    default: mine = bt_scan<16>(fs_row, M, start, end, K, lane, warp); break;
  }
  lists[warp][lane] = mine;
  __syncthreads();
  if (warp != 0) return;
  for (uint32_t w = 1; w < kBtThreads / 32; ++w)
    for (uint32_t e = 0; e < K; ++e) {
      const uint64_t x = lists[w][e];
      if (x == 0) break;
      mine = bt_insert(mine, x, lane);
    }
  const uint32_t n = __popc(__ballot_sync(0xffffffffu, lane < K && mine != 0));
  if (lane == 0) counts[beam] = n;
  if (lane < n) {
    const uint32_t k = ~(uint32_t)mine;
    const float bw = __fdiv_rn(fs, (float)nfft);
    const float yc = __uint_as_float((uint32_t)(mine >> 32));
    const float yl = mag_rn(bin(k - 1)), yr = mag_rn(bin(k + 1));
    float fo = 0.f, rf = __fmul_rn((float)k, bw);
    if (refine == SPX_REFINE_PARABOLIC) {
      const float denom = __fadd_rn(__fsub_rn(yl, __fmul_rn(2.0f, yc)), yr);
      if (fabsf(denom) > 1e-10f) {
        float q = __fdiv_rn(__fmul_rn(0.5f, __fsub_rn(yl, yr)), denom);
        q = fminf(fmaxf(q, -0.5f), 0.5f);
        fo = q;
        rf = __fmul_rn(__fadd_rn((float)k, fo), bw);
      }
    }
    const float2 z = bin(k);
    out[(size_t)beam * K + lane] =
        MaxValueDev{k, z.x, z.y, yc, __fmul_rn(atan2f(z.y, z.x), kRadToDeg), fo, rf, 0u};
  }
}

}  // namespace spx

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
using namespace spx;

struct LaunchSet {  // one FFT launch: its CTA table and cluster size
  BatchCta* d_ctas = nullptr;
  uint32_t n_ctas = 0, cluster = 1, threads = 32, ept = 16;
  size_t smem = 0;
  uint32_t* d_beam_list = nullptr;  // beams of this launch (for the top-K kernel)
  uint32_t n_beams = 0;
};

struct spx_batch {
  int device = 0;
  uint32_t beams = 0, window = 0, K = 8, start = 0, end = 0, refine = 1;
  float fs = 1.0f;
  std::vector<uint32_t> n_point, nfft;
  uint64_t in_total = 0, spec_total = 0;
  BatchBeam* d_beams = nullptr;
  BatchGeom* d_geoms = nullptr;
  float2* d_xch = nullptr;
  uint32_t ept = kEPTDefault, points_per_cta = kPrefLocalCluster;
  LaunchSet all;                       // the single batched launch
  std::vector<LaunchSet> per_size;     // the per-size ("plain") launches
  cudaGraphExec_t graph = nullptr;
  std::vector<void*> allocs;
  ~spx_batch() {
    if (graph) cudaGraphExecDestroy(graph);
    for (void* p : allocs) cudaFree(p);
  }
};

namespace {

template <typename T>
spx_status upload(spx_ctx* ctx, spx_batch* b, const std::vector<T>& v, T** out) {
  *out = nullptr;
  if (v.empty()) return SPX_OK;
  cudaError_t e = cudaMalloc(out, v.size() * sizeof(T));
  if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaMalloc(batch tables)");
  b->allocs.push_back(*out);
  e = cudaMemcpy(*out, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaMemcpy(batch tables)");
  return SPX_OK;
}

// Packs the given beams into clusters of `cl` CTAs (first-fit decreasing by
// group size) and returns the per-CTA table.
std::vector<BatchCta> pack(const std::vector<uint32_t>& ids, const std::vector<uint32_t>& group,
                           uint32_t cl) {
  std::vector<uint32_t> order(ids);
  std::stable_sort(order.begin(), order.end(),
                   [&](uint32_t a, uint32_t b) { return group[a] > group[b]; });
  std::vector<std::vector<uint32_t>> clusters;  // beams per cluster
  std::vector<uint32_t> used;
  for (uint32_t beam : order) {
    const uint32_t gsz = group[beam];
    size_t j = 0;
    while (j < clusters.size() && used[j] + gsz > cl) ++j;
    if (j == clusters.size()) {
      clusters.emplace_back();
      used.push_back(0);
    }
    clusters[j].push_back(beam);
    used[j] += gsz;
  }
  std::vector<BatchCta> ctas;
  ctas.reserve(clusters.size() * cl);
  for (const auto& cb : clusters) {
    uint32_t r = 0;
    for (uint32_t beam : cb)
      for (uint32_t c = 0; c < group[beam]; ++c) ctas.push_back(BatchCta{beam, c, r, 0}), ++r;
    for (; r < cl; ++r) ctas.push_back(BatchCta{kIdle, 0, 0, 0});
  }
  return ctas;
}

spx_status build_launches(spx_ctx* ctx, spx_batch* b) {
  // plans and geometry table with the batch's tuning
  std::map<uint32_t, uint32_t> geom_of;  // nfft -> geometry index
  std::vector<BatchGeom> geoms;
  std::vector<uint32_t> group(b->beams);
  for (uint32_t i = 0; i < b->beams; ++i) {
    const uint32_t n = b->nfft[i];
    if (!geom_of.count(n)) {
      ctx->tuning[n] = {b->ept, b->points_per_cta};
      const FftPlan* plan = nullptr;
      spx_status st = get_plan(ctx, n, &plan);
      if (st != SPX_OK) return st;
      if (plan->big || plan->g.C > kBtMaxC) return fail(ctx, SPX_ERR_UNSUPPORTED, "batch: nfft " + std::to_string(n));
      geom_of[n] = (uint32_t)geoms.size();
      geoms.push_back(BatchGeom{plan->g, plan->d_tw_local, plan->d_tw_cross});
    }
    group[i] = geoms[geom_of[n]].g.C;
  }
  std::vector<BatchBeam> beams(b->beams);
  uint64_t in_off = 0, spec_off = 0;
  for (uint32_t i = 0; i < b->beams; ++i) {
    beams[i] = BatchBeam{in_off, spec_off, b->n_point[i], b->nfft[i], geom_of[b->nfft[i]], 0};
    in_off += b->n_point[i];
    spec_off += (b->nfft[i] + 31u) & ~31u;  // 256-byte aligned spectra
  }
  b->in_total = in_off;
  b->spec_total = spec_off;
  spx_status st = upload(ctx, b, beams, &b->d_beams);
  if (st == SPX_OK) st = upload(ctx, b, geoms, &b->d_geoms);
  if (st != SPX_OK) return st;
  auto make_set = [&](const std::vector<uint32_t>& ids, LaunchSet* ls) -> spx_status {
    uint32_t cl = 1, threads = 32, mpad = 16;
    for (uint32_t id : ids) {
      const FftGeom& g = geoms[geom_of[b->nfft[id]]].g;
      cl = std::max(cl, g.C);
      threads = std::max(threads, g.T);
      mpad = std::max(mpad, g.Mpad);
    }
    std::vector<BatchCta> ctas = pack(ids, group, cl);
    ls->n_ctas = (uint32_t)ctas.size();
    ls->cluster = cl;
    ls->threads = threads;
    ls->ept = b->ept;
    ls->smem = (size_t)mpad * sizeof(float2);
    ls->n_beams = (uint32_t)ids.size();
    // the top-K kernel visits the largest spectra first (outputs are indexed by beam)
    std::vector<uint32_t> by_size(ids);
    std::stable_sort(by_size.begin(), by_size.end(),
                     [&](uint32_t x, uint32_t y) { return b->nfft[x] > b->nfft[y]; });
    spx_status s2 = upload(ctx, b, ctas, &ls->d_ctas);
    if (s2 == SPX_OK) s2 = upload(ctx, b, by_size, &ls->d_beam_list);
    return s2;
  };
  std::vector<uint32_t> all(b->beams);
  for (uint32_t i = 0; i < b->beams; ++i) all[i] = i;
  st = make_set(all, &b->all);
  if (st != SPX_OK) return st;
  std::map<uint32_t, std::vector<uint32_t>> by_size;
  for (uint32_t i = 0; i < b->beams; ++i) by_size[b->nfft[i]].push_back(i);
  b->per_size.clear();
  for (auto& kv : by_size) {
    b->per_size.emplace_back();
    st = make_set(kv.second, &b->per_size.back());
    if (st != SPX_OK) return st;
  }
  return SPX_OK;
}

spx_status launch_set(spx_ctx* ctx, spx_batch* b, const LaunchSet& ls, const void* d_in,
                      spx_max_value* d_out, uint32_t* d_counts) {
  const void* kfn = ls.ept == 32 ? (const void*)fft_batch_kernel<32> : (const void*)fft_batch_kernel<16>;
  cudaError_t e = configure_kernel(kfn, kMaxFftSmem);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "configure fft_batch_kernel");
  const float2* in = static_cast<const float2*>(d_in);
  const BatchBeam* beams = b->d_beams;
  const BatchCta* ctas = ls.d_ctas;
  const BatchGeom* geoms = b->d_geoms;
  uint32_t window = b->window;
  float2* xch = b->d_xch;
  uint32_t ahead = resident_ctas(kfn, ls.threads, ls.smem, ls.cluster);
  void* args[] = {(void*)&in, (void*)&beams, (void*)&ctas, (void*)&geoms,
                  (void*)&window, (void*)&xch, (void*)&ahead};
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(ls.n_ctas, 1, 1);
  cfg.blockDim = dim3(ls.threads, 1, 1);
  cfg.dynamicSmemBytes = ls.smem;
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
  topk_batch_kernel<<<ls.n_beams, kBtThreads, 0, ctx->stream>>>(
      b->d_xch, b->d_beams, b->d_geoms, ls.d_beam_list, b->K, b->start, b->end, b->fs, b->refine,
      reinterpret_cast<MaxValueDev*>(d_out), d_counts);
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
    if (big_size(n)) {  // three-launch transforms: not a cluster of the batch kernel
      delete b;
      return fail(ctx, SPX_ERR_UNSUPPORTED,
                  "spx_batch_create: beam " + std::to_string(i) + " needs nfft " + std::to_string(n) +
                      "; 2^19 and 2^20 points run through spx_fft_peaks, not in a batch");
    }
    b->nfft[i] = n;
  }
  spx_status st = build_launches(ctx, b);
  if (st == SPX_OK) {
    cudaError_t e = cudaMalloc(&b->d_xch, b->spec_total * sizeof(float2));
    if (e == cudaSuccess) b->allocs.push_back(b->d_xch);
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
  if (!d_in || !d_out || !d_counts) return fail(ctx, SPX_ERR_INVALID_ARG, "spx_batch_run: null pointer");
  Guard gd(ctx->device);
  return launch_set(ctx, batch, batch->all, d_in, d_out, d_counts);
}

spx_status spx_batch_run_per_size(spx_ctx* ctx, spx_batch* batch, const void* d_in,
                                  spx_max_value* d_out, uint32_t* d_counts) {
  if (!ctx || !batch) return SPX_ERR_INVALID_ARG;
  if (!d_in || !d_out || !d_counts) return fail(ctx, SPX_ERR_INVALID_ARG, "spx_batch_run_per_size: null pointer");
  Guard gd(ctx->device);
  for (const LaunchSet& ls : batch->per_size) {
    spx_status st = launch_set(ctx, batch, ls, d_in, d_out, d_counts);
    if (st != SPX_OK) return st;
  }
  return SPX_OK;
}

spx_status spx_batch_capture(spx_ctx* ctx, spx_batch* batch, const void* d_in,
                             spx_max_value* d_out, uint32_t* d_counts) {
  if (!ctx || !batch) return SPX_ERR_INVALID_ARG;
  if (!ctx->stream)
    return fail(ctx, SPX_ERR_INVALID_ARG, "spx_batch_capture: set a non-default stream first");
  Guard gd(ctx->device);
  // resolve lazy set-up before capturing
  cudaError_t e = configure_kernel(batch->ept == 32 ? (const void*)fft_batch_kernel<32>
                                                    : (const void*)fft_batch_kernel<16>,
                                   kMaxFftSmem);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "configure fft_batch_kernel");
  e = cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaStreamBeginCapture");
  spx_status st = launch_set(ctx, batch, batch->all, d_in, d_out, d_counts);
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
  if (points_per_thread != 16 && points_per_thread != 32)
    return fail(ctx, SPX_ERR_INVALID_ARG, "spx_batch_tune: points_per_thread must be 16 or 32");
  if (points_per_cta == 0) points_per_cta = kPrefLocalCluster;
  if (points_per_cta < 1024 || points_per_cta > kMaxLocal)
    return fail(ctx, SPX_ERR_INVALID_ARG, "spx_batch_tune: points_per_cta out of range");
  Guard gd(ctx->device);
  batch->ept = points_per_thread;
  batch->points_per_cta = points_per_cta;
  if (batch->graph) {
    cudaGraphExecDestroy(batch->graph);
    batch->graph = nullptr;
  }
  return build_launches(ctx, batch);
}

spx_status spx_batch_autotune(spx_ctx* ctx, spx_batch* batch, const void* d_in,
                              spx_max_value* d_out, uint32_t* d_counts, uint32_t* best_ept,
                              uint32_t* best_points_per_cta) {
  if (!ctx || !batch) return SPX_ERR_INVALID_ARG;
  Guard gd(ctx->device);
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  uint32_t be = batch->ept, bp = batch->points_per_cta;
  for (uint32_t ept : {16u, 32u}) {
    for (uint32_t ppc : {8192u, 16384u}) {
      spx_status st = spx_batch_tune(ctx, batch, ept, ppc);
      if (st != SPX_OK) continue;
      for (int w = 0; w < 2; ++w) st = spx_batch_run(ctx, batch, d_in, d_out, d_counts);
      if (st != SPX_OK) continue;
      cudaEventRecord(e0, ctx->stream);
      for (int r = 0; r < 3; ++r) spx_batch_run(ctx, batch, d_in, d_out, d_counts);
      cudaEventRecord(e1, ctx->stream);
      cudaEventSynchronize(e1);
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      if (ms < best) {
        best = ms;
        be = ept;
        bp = ppc;
      }
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (best_ept) *best_ept = be;
  if (best_points_per_cta) *best_points_per_cta = bp;
  return spx_batch_tune(ctx, batch, be, bp);
}

}  // extern "C"
