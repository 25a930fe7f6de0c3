// fft_kernels.cu — batched windowed, zero-padded C2C FFT with a fused output
// epilogue (complex / |X| / |X|^2 / {|X|, phase}), plus FFT plan building.
//
// Replaces PadDataOp + hipfftExecC2C + MagPhaseOp/MagnitudeOp of the
// reference (include/spectrum/operations/pad_data_op.hpp:82-133,
// src/fft_func/src/fft_processor_rocm.cpp:353-361,
// include/spectrum/operations/magnitude_op.hpp:80-103): the zero padding and
// the window are generated on load, the epilogue runs on the last pass, so
// each beam reads its n_point samples once and writes its spectrum once.
#include <algorithm>
#include <cmath>
#include <map>
#include <mutex>
#include <tuple>
#include <set>
#include <utility>
#include <vector>

#include "fft_core.cuh"
#include "spx_internal.h"

namespace spx {

// ---------------------------------------------------------------------------
// Kernel for nfft <= 16384: one CTA per beam.
// ---------------------------------------------------------------------------
template <int EPT>
__global__ void __launch_bounds__(kMaxLocal / EPT, 1)
fft_out_kernel(const float2* __restrict__ in, uint32_t n_point, const float* __restrict__ win,
               FftGeom g, const float2* __restrict__ tw_local, const float2* __restrict__ tw_cross,
               void* __restrict__ out, uint32_t out_mode, float scale) {
  extern __shared__ float2 s[];
  const uint32_t tid = threadIdx.x, T = blockDim.x;
  const uint32_t beam = blockIdx.x;
  prefetch_future_beam(g, in, n_point, beam, 0, tid, T);
  // C = 1: bin k is element k of the local result, written by the last pass
  local_fft_out<EPT>(s, g, SampleLoader{in + (size_t)beam * n_point, n_point, win}, tw_local, tid, T,
                     BinOut{out, out_mode, scale, &g, beam});
}

// ---------------------------------------------------------------------------
// Kernel for nfft > 16384: one cluster of C CTAs per beam.  The cross-CTA
// exchange goes through device memory instead of distributed shared memory
// (measured on GB300: an L2 round trip moves ~10 TB/s, DSMEM stores ~2 TB/s):
// CTA c writes its C-point DFT outputs into the beam's exchange slot, a
// cluster barrier (release/acquire) publishes them, CTA k1 reads row k1 in
// its first Stockham pass and then invalidates the row's L2 lines
// (discard.global.L2), so the slot never costs a DRAM write-back and only
// the slots of clusters in flight occupy L2.
// ---------------------------------------------------------------------------
template <int EPT>
__global__ void __launch_bounds__(kMaxLocal / EPT, 1)
fft_xl_kernel(const float2* __restrict__ in, uint32_t n_point, const float* __restrict__ win,
              FftGeom g, const float2* __restrict__ tw_local, const float2* __restrict__ tw_cross,
              float2* __restrict__ xch) {
  extern __shared__ float2 s[];
  cg::cluster_group cl = cg::this_cluster();
  const uint32_t tid = threadIdx.x, T = blockDim.x;
  const uint32_t c = cl.block_rank();
  const uint32_t beam = blockIdx.x / g.C;
  float2* slot = xch + (size_t)beam * g.nfft;
  const SampleLoader ld{in + (size_t)beam * n_point, n_point, win};
  prefetch_future_beam(g, in, n_point, beam, c, tid, T);
  switch (g.C) {
    case 2: cross_stage_exchange<2>(slot, c, g.M, ld, tw_cross, tid, T); break;
    case 3: cross_stage_exchange<3>(slot, c, g.M, ld, tw_cross, tid, T); break;
    case 4: cross_stage_exchange<4>(slot, c, g.M, ld, tw_cross, tid, T); break;
    case 6: cross_stage_exchange<6>(slot, c, g.M, ld, tw_cross, tid, T); break;
    case 8: cross_stage_exchange<8>(slot, c, g.M, ld, tw_cross, tid, T); break;
    case 9: cross_stage_exchange<9>(slot, c, g.M, ld, tw_cross, tid, T); break;
    case 12: cross_stage_exchange<12>(slot, c, g.M, ld, tw_cross, tid, T); break;
    default: cross_stage_exchange<16>(slot, c, g.M, ld, tw_cross, tid, T); break;
  }
  cl.sync();
  float2* row = slot + (size_t)c * g.M;
  // row c was read by this CTA alone: it takes the CTA's spectrum row
  // (row[i] = X[c + C*i]); rows_transpose_kernel writes the output
  if (EPT != 16 || !ct_menu_fft<0>(g.M, s, ExchangeLoader{row}, tw_local, tid, RowOut{row}))
    local_fft_out<EPT>(s, g, ExchangeLoader{row}, tw_local, tid, T, RowOut{row});
}

// The same transform as fft_xl_kernel for power-of-two local sizes M (M / 16
// threads) and C in {2, 4, 8, 16}, on all SMs: a persistent cooperative
// launch of G groups of C CTAs (one CTA per SM for M = 16384), group q
// transforming beams q, q + G, ...; a bounded device-memory barrier per beam
// (group_barrier) replaces the cluster barrier (clusters of 8 one-SM CTAs fit
// on 120 of the 152 SMs).  Each CTA leaves its spectrum row in the beam's
// exchange slot; rows_transpose_kernel then writes the output (the stride-C
// stores of a direct epilogue cost more than the extra pass: 0.332 vs 0.313 ms
// for 256 x 131072 points).
template <int M>
__global__ void __launch_bounds__(M / 16, 16384 / M)
fft_group_out_kernel(const float2* __restrict__ in, uint32_t n_point, const float* __restrict__ win,
                     FftGeom g, const float2* __restrict__ tw_local, const float2* __restrict__ tw_cross,
                     float2* __restrict__ xch, uint32_t* __restrict__ arrive, uint32_t* __restrict__ err,
                     uint32_t groups) {
  extern __shared__ float2 s[];
  constexpr uint32_t T = M / 16;
  const uint32_t tid = threadIdx.x;
  const uint32_t grp = blockIdx.x / g.C, c = blockIdx.x - grp * g.C;
#pragma unroll 1
  for (uint32_t beam = grp; beam < g.beams; beam += groups) {
    float2* slot = xch + (size_t)beam * g.nfft;
    const SampleLoader ld{in + (size_t)beam * n_point, n_point, win};
    prefetch_future_beam(g, in, n_point, beam, c, tid, T);
    switch (g.C) {
      case 2: cross_stage_exchange<2>(slot, c, M, ld, tw_cross, tid, T); break;
      case 4: cross_stage_exchange<4>(slot, c, M, ld, tw_cross, tid, T); break;
      case 8: cross_stage_exchange<8>(slot, c, M, ld, tw_cross, tid, T); break;
      default: cross_stage_exchange<16>(slot, c, M, ld, tw_cross, tid, T); break;
    }
    group_barrier(arrive + beam, g.C, err);
    float2* row = slot + (size_t)c * M;
    // row c was read by this CTA alone: it takes the CTA's spectrum row
    // (row[i] = X[c + C*i]) from the last pass's registers;
    // rows_transpose_kernel writes the output
    ct_local_fft_out<M>(s, ExchangeLoader{row}, tw_local, tid, RowOut{row});
  }  // (the next beam's group barrier orders these reads of s before its local FFT)
}

// Bins k1 + C*q of the output from the row layout rows[beam][k1][q] (C rows
// of M columns per beam, C <= 128): one CTA per `tc` columns of one beam; the
// tile comes in along the rows (contiguous runs) and goes out in bin order
// (contiguous runs in every output mode but the mirrored ones), through
// shared memory with a row pitch of tc + 1 (conflict-free both ways).
__global__ void __launch_bounds__(256)
rows_transpose_kernel(FftGeom g, const float2* __restrict__ rows, uint32_t tc, uint32_t cmagic,
                      void* __restrict__ out, uint32_t out_mode, float scale, uint32_t beam0) {
  extern __shared__ float2 tile[];  // [C][tc + 1]
  const uint32_t tid = threadIdx.x, C = g.C, M = g.M, ld = tc + 1;
  const uint32_t beam = beam0 + blockIdx.y, q0 = blockIdx.x * tc;
  const uint32_t tshift = 31u - __clz(tc);  // tc is a power of two
  const float2* src = rows + (size_t)beam * g.nfft + q0;
  for (uint32_t f = tid; f < C * tc; f += 256) {
    const uint32_t r = f >> tshift, q = f & (tc - 1);
    if (q0 + q < M) tile[r * ld + q] = __ldcs(src + (size_t)r * M + q);
  }
  __syncthreads();
  const uint32_t k0 = C * q0;
  for (uint32_t e = tid; e < C * tc; e += 256) {
    const uint32_t q = __umulhi(e, cmagic), k1 = e - q * C;  // e div C, e mod C
    if (q0 + q < M) store_bin(out, out_mode, scale, g, beam, k0 + e, tile[k1 * ld + q]);
  }
}

spx_status launch_rows_transpose(spx_ctx* ctx, const FftGeom& g, const float2* rows, uint32_t beams,
                                 void* d_out, uint32_t out_mode, float scale) {
  uint32_t tc = 32;
  while (g.C * tc < 1024) tc *= 2;
  const uint32_t cmagic = 0xFFFFFFFFu / g.C + 1u;  // e div C = umulhi(e, cmagic) for e * C < 2^32
  const size_t smem = (size_t)g.C * (tc + 1) * sizeof(float2);
  constexpr uint32_t kMaxGridY = 65535;  // beams per launch (gridDim.y)
  for (uint32_t b0 = 0; b0 < beams; b0 += kMaxGridY) {
    const dim3 grid((g.M + tc - 1) / tc, std::min(beams - b0, kMaxGridY));
    rows_transpose_kernel<<<grid, 256, smem, ctx->stream>>>(g, rows, tc, cmagic, d_out, out_mode, scale, b0);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(ctx, e, "launch rows_transpose_kernel");
  }
  return SPX_OK;
}

bool group_geometry(const FftGeom& g) {
  return g.C > 1 && (g.C & (g.C - 1)) == 0 && g.ept == 16 && (g.M == 4096 || g.M == 8192 || g.M == 16384) &&
         g.T == g.M / 16;
}

// ---------------------------------------------------------------------------
// Host: geometry and twiddle tables.
// ---------------------------------------------------------------------------
bool is_smooth23(uint32_t n) {
  if (n == 0) return false;
  while (n % 2 == 0) n /= 2;
  while (n % 3 == 0) n /= 3;
  return n == 1;
}

bool build_geom(uint32_t nfft, FftGeom* g, uint32_t ept, uint32_t pref_local) {
  if (nfft < 2 || !is_smooth23(nfft)) return false;
  if (ept != 16 && ept != 32) return false;
  if (pref_local < 1024 || pref_local > kMaxLocal) return false;
  // C = 1 up to kMaxLocal points; beyond, the smallest cluster whose CTAs
  // hold <= kPrefLocalCluster points (two CTAs per SM), else <= kMaxLocal.
  static const uint32_t kClusters[] = {2, 3, 4, 6, 8, 9, 12, 16};
  uint32_t C = nfft <= kMaxLocal ? 1u : 0u;
  for (uint32_t lim : {pref_local, kMaxLocal}) {
    for (uint32_t c : kClusters) {
      if (C == 0 && nfft % c == 0 && nfft / c <= lim) C = c;
    }
  }
  if (C == 0) return false;
  FftGeom r{};
  r.nfft = nfft;
  r.C = C;
  r.M = nfft / C;
  r.Mpad = sw_len(r.M);
  uint32_t a = 0, b = 0, m = r.M;
  while (m % 2 == 0) { m /= 2; ++a; }
  while (m % 3 == 0) { m /= 3; ++b; }
  std::vector<uint32_t> rad;
  while (a >= 4) { rad.push_back(16); a -= 4; }
  uint32_t rem2 = 1u << a;  // 1, 2, 4 or 8
  if (rem2 == 8) { rad.insert(rad.begin(), 8); rem2 = 1; }
  while (b >= 2) { rad.push_back(9); b -= 2; }
  if (b == 1) rad.push_back(3);
  if (rem2 > 1) rad.push_back(rem2);
  if (rad.empty()) rad.push_back(1);  // M == 1 cannot happen for nfft >= 2 with C <= nfft/2
  if (rad.size() > (size_t)kMaxPass) return false;
  r.npass = (uint32_t)rad.size();
  uint32_t Ns = 1, off = 0;
  for (uint32_t p = 0; p < r.npass; ++p) {
    r.radix[p] = rad[p];
    r.ns[p] = Ns;
    r.twoff[p] = off;
    r.nsmagic[p] = Ns > 1 ? (uint32_t)(((1ull << 32) + Ns - 1) / Ns) : 0u;
    off += tw_entries(rad[p], Ns);
    Ns *= rad[p];
  }
  uint32_t T = (r.M + ept - 1) / ept;
  T = ((T + 31u) / 32u) * 32u;
  if (T < 32) T = 32;
  if (T > kMaxLocal / ept) return false;
  r.T = T;
  r.ept = ept;
  *g = r;
  return true;
}

// exp(-2 pi i m / L) in FP64, rounded to FP32.
static inline float2 twiddle(uint64_t m, uint64_t L) {
  m %= L;
  const double a = -2.0 * M_PI * (double)m / (double)L;
  return make_float2((float)std::cos(a), (float)std::sin(a));
}

void fill_local_twiddles(const FftGeom& g, float2* twl) {
  for (uint32_t p = 0; p < g.npass; ++p) {
    const uint32_t R = g.radix[p], Ns = g.ns[p];
    const uint64_t L = (uint64_t)Ns * R;
    if (tw_split(R, Ns)) {
      for (uint32_t l = 0; l < 64; ++l) twl[g.twoff[p] + l] = twiddle(l, L);
      for (uint32_t j = 0; j < (Ns + 63) / 64; ++j) twl[g.twoff[p] + 64 + j] = twiddle(64ull * j, L);
      continue;
    }
    for (uint32_t r = 1; r <= tw_rows(R); ++r)
      for (uint32_t k = 0; k < Ns; ++k) twl[g.twoff[p] + (r - 1) * Ns + k] = twiddle((uint64_t)r * k, L);
  }
}

FftPlan::~FftPlan() {
  if (d_tw_local) cudaFree(d_tw_local);
  if (d_tw_cross) cudaFree(d_tw_cross);
  if (d_chirp) cudaFree(d_chirp);
  if (d_bfft) cudaFree(d_bfft);
}

spx_status get_plan(spx_ctx* ctx, uint32_t nfft, const FftPlan** out) {
  auto te = ctx->tuning.find(nfft);
  const uint32_t ept = te != ctx->tuning.end() ? te->second.first : (uint32_t)kEPTDefault;
  const uint32_t pref = te != ctx->tuning.end() ? te->second.second : kPrefLocalCluster;
  const uint64_t key = ((uint64_t)ept << 56) | ((uint64_t)pref << 32) | nfft;
  auto it = ctx->plans.find(key);
  if (it != ctx->plans.end()) {
    *out = it->second.get();
    return SPX_OK;
  }
  auto plan = std::make_unique<FftPlan>();
  if (big_size(nfft)) {
    spx_status st = build_big_plan(ctx, nfft, plan.get());
    if (st != SPX_OK) return st;
    *out = plan.get();
    ctx->plans.emplace(key, std::move(plan));
    return SPX_OK;
  }
  if (huge_size(nfft)) {
    spx_status st = build_huge_plan(ctx, nfft, plan.get());
    if (st != SPX_OK) return st;
    *out = plan.get();
    ctx->plans.emplace(key, std::move(plan));
    return SPX_OK;
  }
  if (!build_geom(nfft, &plan->g, ept, pref)) {
    if (!bluestein_size(nfft))
      return fail(ctx, SPX_ERR_INVALID_ARG,
                  "nfft=" + std::to_string(nfft) +
                      " is not a supported size (any length 2 .. 2^27; 2^a*3^b up to 2^28 with a split into"
                      " two factors <= 16384)");
    spx_status st = build_bluestein_plan(ctx, nfft, plan.get());
    if (st != SPX_OK) return st;
    *out = plan.get();
    ctx->plans.emplace(key, std::move(plan));
    return SPX_OK;
  }
  const FftGeom& g = plan->g;
  std::vector<float2> twl(std::max<uint32_t>(g.M, 1));
  fill_local_twiddles(g, twl.data());
  cudaError_t e = cudaMalloc(&plan->d_tw_local, twl.size() * sizeof(float2));
  if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaMalloc(twiddles)");
  e = cudaMemcpy(plan->d_tw_local, twl.data(), twl.size() * sizeof(float2), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaMemcpy(twiddles)");
  if (g.C > 1) {  // W_N^{n2}, n2 < M: the cross stage raises it to W_N^{n2 k1}
    std::vector<float2> twc((size_t)g.M);
    for (uint32_t n2 = 0; n2 < g.M; ++n2) twc[n2] = twiddle((uint64_t)n2, g.nfft);
    e = cudaMalloc(&plan->d_tw_cross, twc.size() * sizeof(float2));
    if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaMalloc(cross twiddles)");
    e = cudaMemcpy(plan->d_tw_cross, twc.data(), twc.size() * sizeof(float2), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaMemcpy(cross twiddles)");
  }
  *out = plan.get();
  ctx->plans.emplace(key, std::move(plan));
  return SPX_OK;
}

// The window table of one (window, n_point): w[n] = window_at(n) (fft_core.cuh),
// the evaluation the uneven batch makes per sample.
__global__ void window_table_kernel(uint32_t window, uint32_t n_point, float* __restrict__ w) {
  const WindowGen g = make_window_gen(window, n_point);
  for (uint32_t n = blockIdx.x * blockDim.x + threadIdx.x; n < n_point; n += gridDim.x * blockDim.x)
    w[n] = window_at(g, n);
}

spx_status get_window(spx_ctx* ctx, uint32_t window, uint32_t n_point, const float** out) {
  if (window == SPX_WINDOW_NONE) {
    *out = nullptr;
    return SPX_OK;
  }
  if (window > SPX_WINDOW_BLACKMAN_HARRIS)
    return fail(ctx, SPX_ERR_INVALID_ARG, "unknown window type " + std::to_string(window));
  const uint64_t key = ((uint64_t)window << 32) | n_point;
  auto it = ctx->windows.find(key);
  if (it != ctx->windows.end()) {
    *out = it->second;
    return SPX_OK;
  }
  float* d = nullptr;
  cudaError_t e = cudaMalloc(&d, std::max<size_t>(1, n_point) * sizeof(float));
  if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaMalloc(window)");
  const uint32_t blocks = std::min<uint32_t>((n_point + 255) / 256, 4096);
  window_table_kernel<<<std::max(blocks, 1u), 256, 0, ctx->stream>>>(window, n_point, d);
  e = cudaGetLastError();
  // filled once per (window, n_point); later calls may come on another stream
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) {
    cudaFree(d);
    return cuda_fail(ctx, e, "window table");
  }
  ctx->windows[key] = d;
  *out = d;
  return SPX_OK;
}

// ---------------------------------------------------------------------------
// Host: launch.
// ---------------------------------------------------------------------------
// Raises the dynamic shared-memory limit and allows clusters of 9 and 16
// once per (device, kernel).
cudaError_t configure_kernel(const void* kernel, size_t max_smem) {
  static std::mutex mu;
  static std::set<std::pair<int, const void*>> done;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> lock(mu);
  if (done.count({dev, kernel})) return cudaSuccess;
  e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)max_smem);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  if (e != cudaSuccess) return e;
  done.insert({dev, kernel});
  return cudaSuccess;
}

// CTAs of a launch of `kernel` resident at once (blocks per SM times SMs,
// or active clusters times the cluster size), cached per (device, kernel,
// shape): the L2 prefetch distance of the FFT kernels.
uint32_t resident_ctas(const void* kernel, uint32_t threads, size_t smem, uint32_t cluster) {
  static std::mutex mu;
  static std::map<std::tuple<int, const void*, uint32_t, uint32_t, size_t>, uint32_t> cache;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  const auto key = std::make_tuple(dev, kernel, threads, cluster, smem);
  {
    std::lock_guard<std::mutex> lock(mu);
    auto it = cache.find(key);
    if (it != cache.end()) return it->second;
  }
  uint32_t n = 0;
  if (cluster <= 1) {
    int per_sm = 0, sms = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, (int)threads, smem) == cudaSuccess &&
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess)
      n = (uint32_t)(per_sm * sms);
  } else {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(cluster, 1, 1);
    cfg.blockDim = dim3(threads, 1, 1);
    cfg.dynamicSmemBytes = smem;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = cluster;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int clusters = 0;
    if (cudaOccupancyMaxActiveClusters(&clusters, kernel, &cfg) == cudaSuccess) n = (uint32_t)clusters * cluster;
  }
  cudaGetLastError();
  std::lock_guard<std::mutex> lock(mu);
  cache[key] = n;
  return n;
}

uint32_t resident_beams(const void* kernel, const FftGeom& g, size_t smem) {
  return resident_ctas(kernel, g.T, smem, g.C) / g.C;
}

template <typename K>
static cudaError_t launch_beams(K kernel, FftGeom& g, uint32_t beams, size_t smem,
                                cudaStream_t stream, void** args, bool prefetch) {
  cudaError_t e0 = configure_kernel((const void*)kernel, kMaxFftSmem);
  if (e0 != cudaSuccess) return e0;
  g.beams = beams;
  g.ahead = prefetch ? resident_beams((const void*)kernel, g, smem) : 0u;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(beams * g.C, 1, 1);
  cfg.blockDim = dim3(g.T, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = stream;
  cudaLaunchAttribute attr[1];
  if (g.C > 1) {
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = g.C;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
  }
  return cudaLaunchKernelExC(&cfg, (const void*)kernel, args);
}

spx_status launch_fft_out(spx_ctx* ctx, const FftPlan& plan, const float2* d_in,
                          uint32_t beams, uint32_t n_point, const float* d_win,
                          uint32_t out_mode, float scale, void* d_out) {
  if (beams == 0) return SPX_OK;
  if (plan.big) return launch_fft_big(ctx, plan, d_in, beams, n_point, d_win, out_mode, scale, d_out);
  if (plan.bluestein) return launch_fft_bluestein(ctx, plan, d_in, beams, n_point, d_win, out_mode, scale, d_out);
  if (plan.huge) return launch_fft_huge(ctx, plan, d_in, beams, n_point, d_win, out_mode, scale, d_out);
  FftGeom g = plan.g;
  const float2* twl = plan.d_tw_local;
  const float2* twc = plan.d_tw_cross;
  const size_t smem = (size_t)g.Mpad * sizeof(float2);
  cudaError_t e;
  const bool wide = g.ept == 32;
  if (g.C == 1) {
    void* args[] = {(void*)&d_in, (void*)&n_point, (void*)&d_win, (void*)&g,
                    (void*)&twl,  (void*)&twc,     (void*)&d_out, (void*)&out_mode,
                    (void*)&scale};
    e = wide ? launch_beams(fft_out_kernel<32>, g, beams, smem, ctx->stream, args, !ctx->input_on_host)
             : launch_beams(fft_out_kernel<16>, g, beams, smem, ctx->stream, args, !ctx->input_on_host);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "launch fft_out_kernel");
    return SPX_OK;
  }
  const size_t xch_bytes = ((size_t)beams * g.nfft * sizeof(float2) + 255) & ~(size_t)255;
  void* xch = nullptr;
  spx_status st = get_scratch(ctx, kSlotExchange, xch_bytes + (size_t)beams * sizeof(uint32_t), &xch);
  if (st != SPX_OK) return st;
  float2* xchp = static_cast<float2*>(xch);
  if (group_geometry(g)) {
    uint32_t* arrive = reinterpret_cast<uint32_t*>(static_cast<char*>(xch) + xch_bytes);
    e = cudaMemsetAsync(arrive, 0, (size_t)beams * sizeof(uint32_t), ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaMemsetAsync(group barriers)");
    const void* kfn = g.M == 16384 ? (const void*)fft_group_out_kernel<16384>
                      : g.M == 8192 ? (const void*)fft_group_out_kernel<8192>
                                    : (const void*)fft_group_out_kernel<4096>;
    e = configure_kernel(kfn, kMaxFftSmem);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "configure fft_group_out_kernel");
    uint32_t groups = resident_ctas(kfn, g.T, smem, 1) / g.C;  // all resident at once (cooperative)
    if (groups > beams) groups = beams;
    if (groups == 0) return fail(ctx, SPX_ERR_CUDA, "fft_group_out_kernel: a group of CTAs does not fit the device");
    g.beams = beams;
    g.ahead = ctx->input_on_host ? 0u : groups;
    uint32_t* err = ctx->d_error;
    void* gargs[] = {(void*)&d_in, (void*)&n_point, (void*)&d_win, (void*)&g,   (void*)&twl,
                     (void*)&twc,  (void*)&xchp,    (void*)&arrive, (void*)&err, (void*)&groups};
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
    e = cudaLaunchKernelExC(&cfg, kfn, gargs);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "launch fft_group_out_kernel");
    return launch_rows_transpose(ctx, g, xchp, beams, d_out, out_mode, scale);
  }
  void* args[] = {(void*)&d_in, (void*)&n_point, (void*)&d_win, (void*)&g,
                  (void*)&twl,  (void*)&twc,     (void*)&xchp};
  e = wide ? launch_beams(fft_xl_kernel<32>, g, beams, smem, ctx->stream, args, !ctx->input_on_host)
           : launch_beams(fft_xl_kernel<16>, g, beams, smem, ctx->stream, args, !ctx->input_on_host);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "launch fft_xl_kernel");
  return launch_rows_transpose(ctx, g, xchp, beams, d_out, out_mode, scale);
}

}  // namespace spx
