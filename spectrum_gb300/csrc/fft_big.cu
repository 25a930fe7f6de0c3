// fft_big.cu — transforms of 2^19, 2^20 and 2^21 points (the precision
// workload's 2^20-point beams; 2^21 = the reference's nextPow2(2^20) x
// repeat_count 2), beyond what one cluster holds on chip.
//
// nfft = Cb * M, n = M*n1 + n2, k = k1 + Cb*k2:
//   launch 1 (big_cols_kernel; big_cols_pipe_kernel for 2^19): for each n2,
//     the Cb-point DFT over n1 of the windowed, zero-padded samples, times
//     W_N^{n2 k1}, written to scratch[beam][k1][n2] (device memory);
//   2^19 and 2^20 (M = 4096, Cb = 128 or 256): launch 2 (big_rows4_kernel)
//     transforms four rows k1 = 4r .. 4r+3 per CTA and writes bins
//     4r .. 4r+3 + Cb*k2 of the output in the requested mode: runs of four
//     bins, one 32-byte sector, so no separate reordering pass;
//   2^21 (M = 16384, Cb = 128): launch 2 (big_rows_kernel) transforms row k1
//     and writes X[k1 + Cb*k2] back over the row it read; launch 3
//     (rows_transpose_kernel, fft_kernels.cu) writes bin order in the
//     requested mode in contiguous runs (a 16384-point row per CTA leaves no
//     room for four rows, and stride-Cb stores straight from the row kernel
//     kept its SMs waiting on the store queue: 0.63 ms for 64 x 2^20 points).
// All twiddles are FP64-generated and stored in FP32, which is what the
// 120 dB dynamic range of the precision workload needs: W_N^{n2 k1}, k1 =
// a + 16 b, as the product of two factor tables [a][n2] = W_N^{n2 a} and
// [b][n2] = W_N^{16 n2 b} (a warp's 32 columns read 256 contiguous bytes of
// each; a CTA's slice of the second, 4 KB, is read by all its warps from L1,
// where the full [k1][n2] table of nfft entries came from L2: 64 x 2^20
// 0.591 -> 0.580 ms, 128 x 2^19 0.479 -> 0.460 ms, max error vs FP64
// 2.3e-7 -> 2.2e-7 of the peak); W_M from the local plan.  Replaces hipFFT's internal
// multi-pass plan for large sizes (src/fft_func/src/fft_processor_rocm.cpp:176-193).
#include <algorithm>
#include <cmath>
#include <vector>

#include "fft_core.cuh"
#include "spx_internal.h"

namespace spx {

constexpr uint32_t kBigM = 16384;     // row length of the 2^21-point transform
constexpr uint32_t kBigM4 = 4096;     // row length of the 2^19 / 2^20-point transforms
constexpr uint32_t kRows4 = 4;        // rows per CTA of big_rows4_kernel

// Row length M of a big transform of nfft points.
static uint32_t big_rows(uint32_t nfft) { return nfft <= (1u << 20) ? kBigM4 : kBigM; }

// One CTA = 32 consecutive n2 columns x Cb rows (n1); lane = column, warp
// t < G = row group (every warp access is 32 consecutive columns of one row:
// 256-byte global runs, conflict-free shared rows); rows of M points.
// Cb = G x J: stage 1 is the J-point DFT over rows t + G j, on samples loaded
// straight into registers (J loads in flight per thread); the shared tile
// [Cb][32] only carries stage 1's outputs to stage 2, the G-point DFT over t.
template <int CB, int G>
__global__ void __launch_bounds__(32 * G)
big_cols_kernel(const float2* __restrict__ in, uint32_t n_point, const float* __restrict__ win,
                const float2* __restrict__ twN, uint32_t nfft, float2* __restrict__ scratch,
                uint32_t ahead, uint32_t M) {
  extern __shared__ float2 tile_raw[];
  float2(*tile)[32] = reinterpret_cast<float2(*)[32]>(tile_raw);  // [CB][32]
  const uint32_t tid = threadIdx.x;
  const uint32_t beam = blockIdx.y, n2_0 = blockIdx.x * 32;
  const float2* x = in + (size_t)beam * n_point;
  {  // L2 prefetch of the 32-column tile of the CTA `ahead` places later
    const uint64_t f = (uint64_t)blockIdx.y * gridDim.x + blockIdx.x + ahead;
    if (ahead && f < (uint64_t)gridDim.x * gridDim.y && tid < CB) {
      const uint32_t fb = (uint32_t)(f / gridDim.x), fc = (uint32_t)(f % gridDim.x) * 32;
      const uint32_t lo = tid * M + fc, hi = min(lo + 32, n_point);
      if (lo < hi) prefetch_l2(in + (size_t)fb * n_point + lo, (size_t)(hi - lo) * sizeof(float2), 0, 1);
    }
  }
  const uint32_t col = tid & 31, t = tid >> 5;
  constexpr int J = CB / G;  // stage-1 radix
  static_assert(J == 16, "the W_N factor tables are built for k1 = a + 16 b");
  // stage 1: thread t transforms rows t + G j (j < J), twiddles W_CB^{t a}
  float2 v[J];
#pragma unroll
  for (int j = 0; j < J; ++j) v[j] = load_sample(x, (t + G * j) * M + n2_0 + col, n_point, win);
  Dft<J>::run(v);
#pragma unroll
  for (int a = 1; a < J; ++a) {
    const uint32_t e = (t * a) % CB;
    v[a] = cmul(v[a], __ldg(twN + (size_t)(J + G) * M + e));  // W_CB^e, after the two factor tables
  }
#pragma unroll
  for (int a = 0; a < J; ++a) tile[t + G * a][col] = v[a];
  __syncthreads();
  // stage 2: for a = t, t + G, ... (< J), the G-point DFT over t' of rows t' + G a -> k1 = a + J b
#pragma unroll
  for (uint32_t a = t; a < (uint32_t)J; a += G) {
    float2 w[G];
#pragma unroll
    for (int tp = 0; tp < G; ++tp) w[tp] = tile[tp + G * a][col];
    Dft<G>::run(w);
    const uint32_t n2 = n2_0 + col;
    float2* o = scratch + (size_t)beam * nfft + n2;
    const float2 ta = __ldg(twN + (size_t)a * M + n2);  // W_N^{n2 a}
#pragma unroll
    for (int b = 0; b < G; ++b) {
      const uint32_t k1 = a + J * b;  // W_N^{n2 k1} = W_N^{n2 a} W_N^{n2 J b}
      o[(size_t)k1 * M] = cmul(w[b], cmul(ta, __ldg(twN + (size_t)(J + b) * M + n2)));
    }
  }
}

// 8-byte asynchronous copy global -> shared (zero-filled when src_bytes is 0).
SPX_DEV void cp_async8(void* dst, const void* src, uint32_t src_bytes) {
  const uint32_t d = (uint32_t)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;" ::"r"(d), "l"(src), "r"(src_bytes) : "memory");
}
SPX_DEV void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
SPX_DEV void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// The column DFTs of big_cols_kernel in a persistent loop over the tiles
// f = blockIdx.x, blockIdx.x + gridDim.x, ... (beam f / tpb, columns
// 32 (f mod tpb) ..): while a CTA transforms tile f, the samples of its next
// tile stream into shared memory by asynchronous copies.  Each thread copies
// exactly the elements it reads itself (rows t + G j of its column), so the
// landing buffer needs no barrier; stage 1's outputs alternate between two
// exchange tiles, so one CTA barrier per tile orders every access.  The
// arithmetic is big_cols_kernel's: the same bits.
template <int CB, int G>
__global__ void __launch_bounds__(32 * G, 2)
big_cols_pipe_kernel(const float2* __restrict__ in, uint32_t n_point, const float* __restrict__ win,
                     const float2* __restrict__ twN, uint32_t nfft, float2* __restrict__ scratch, uint32_t M,
                     uint32_t tpb, uint32_t total) {
  extern __shared__ float2 tile_raw[];
  float2(*land)[32] = reinterpret_cast<float2(*)[32]>(tile_raw);                 // [CB][32]
  float2(*xch0)[32] = reinterpret_cast<float2(*)[32]>(tile_raw + CB * 32);       // [CB][32]
  float2(*xch1)[32] = reinterpret_cast<float2(*)[32]>(tile_raw + 2 * CB * 32);   // [CB][32]
  constexpr int J = CB / G;  // stage-1 radix
  static_assert(J == 16, "the W_N factor tables are built for k1 = a + 16 b");
  const uint32_t tid = threadIdx.x, col = tid & 31, t = tid >> 5;
  auto issue = [&](uint32_t f) {  // this thread's samples of tile f into its landing slots
    const uint32_t beam = f / tpb, n2_0 = (f - beam * tpb) * 32;
    const float2* x = in + (size_t)beam * n_point;
#pragma unroll
    for (int j = 0; j < J; ++j) {
      const uint32_t n = (t + G * j) * M + n2_0 + col;
      const bool ok = n < n_point;
      cp_async8(&land[t + G * j][col], ok ? x + n : x, ok ? 8u : 0u);
    }
    cp_async_commit();
  };
  uint32_t f = blockIdx.x;
  if (f < total) issue(f);
  for (uint32_t it = 0; f < total; ++it, f += gridDim.x) {
    const uint32_t beam = f / tpb, n2_0 = (f - beam * tpb) * 32;
    cp_async_wait_all();  // this thread's copies of tile f have landed
    float2 v[J];
#pragma unroll
    for (int j = 0; j < J; ++j) v[j] = land[t + G * j][col];
    if (win) {  // window of the samples inside the beam (load_sample's arithmetic)
#pragma unroll
      for (int j = 0; j < J; ++j) {
        const uint32_t n = (t + G * j) * M + n2_0 + col;
        if (n < n_point) {
          const float w = __ldg(win + n);
          v[j].x = __fmul_rn(v[j].x, w);
          v[j].y = __fmul_rn(v[j].y, w);
        }
      }
    }
    Dft<J>::run(v);
#pragma unroll
    for (int a = 1; a < J; ++a) {
      const uint32_t e = (t * a) % CB;
      v[a] = cmul(v[a], __ldg(twN + (size_t)(J + G) * M + e));  // W_CB^e
    }
    float2(*xch)[32] = (it & 1u) ? xch1 : xch0;
#pragma unroll
    for (int a = 0; a < J; ++a) xch[t + G * a][col] = v[a];
    // the stores above depend on every landed value, so this thread's reads
    // of its landing slots are complete before the slots are refilled
    if (f + gridDim.x < total) issue(f + gridDim.x);
    __syncthreads();
    const uint32_t n2 = n2_0 + col;
    float2* o = scratch + (size_t)beam * nfft + n2;
#pragma unroll
    for (uint32_t a = t; a < (uint32_t)J; a += G) {
      float2 w[G];
#pragma unroll
      for (int tp = 0; tp < G; ++tp) w[tp] = xch[tp + G * a][col];
      Dft<G>::run(w);
      const float2 ta = __ldg(twN + (size_t)a * M + n2);  // W_N^{n2 a}
#pragma unroll
      for (int b = 0; b < G; ++b) {
        const uint32_t k1 = a + J * b;  // W_N^{n2 k1} = W_N^{n2 a} W_N^{n2 J b}
        o[(size_t)k1 * M] = cmul(w[b], cmul(ta, __ldg(twN + (size_t)(J + b) * M + n2)));
      }
    }
  }
}

template <int EPT>
__global__ void __launch_bounds__(kMaxLocal / EPT, 1)
big_rows_kernel(FftGeom g, const float2* __restrict__ tw_local, float2* __restrict__ scratch) {
  extern __shared__ float2 s[];
  const uint32_t tid = threadIdx.x, T = blockDim.x;
  const uint32_t beam = blockIdx.x / g.C, k1 = blockIdx.x % g.C;
  float2* row = scratch + (size_t)beam * g.nfft + (size_t)k1 * g.M;
  if (g.ahead && blockIdx.x + g.ahead < gridDim.x)  // the row the CTA one wave later reads
    prefetch_l2(row + (size_t)g.ahead * g.M, (size_t)g.M * sizeof(float2), tid, T);
  // the row was read by this CTA alone (first pass, before its barrier)
  if constexpr (EPT == 16) {
    if (g.M == 16384 && T == 1024) {  // the last pass writes the row from its registers
      ct_local_fft_out<16384>(s, SampleLoader{row, g.M, nullptr}, tw_local, tid, RowOutStream{row});
      return;
    }
  }
  local_fft<EPT>(s, g, SampleLoader{row, g.M, nullptr}, tw_local, tid, T);
  for (uint32_t i = tid; i < g.M; i += T) __stcs(row + i, s[sw(i)]);
}

// Four rows k1 = r0 .. r0+3 of 4096 points per CTA (four groups of 256
// threads, one row each, in shared memory rows kRowPad4 elements apart), then
// the bins r0 + q + Cb*k2 (q < 4) in the requested mode: each run of four
// bins is one 32-byte sector of the output.  The row pitch puts the four rows
// of one k2 on different bank pairs for a half-warp's reads.
constexpr uint32_t kRowPad4 = sw_len(kBigM4) + 4;

__global__ void __launch_bounds__(kRows4 * 256, 1)
big_rows4_kernel(FftGeom g, const float2* __restrict__ tw_local, const float2* __restrict__ scratch,
                 void* __restrict__ out, uint32_t out_mode, float scale) {
  extern __shared__ float2 s[];
  constexpr uint32_t TG = 256;
  const uint32_t tid = threadIdx.x, grp = tid / TG;
  const uint32_t per_beam = g.C / kRows4;
  const uint32_t beam = blockIdx.x / per_beam, r0 = (blockIdx.x - beam * per_beam) * kRows4;
  const float2* row = scratch + (size_t)beam * g.nfft + (size_t)(r0 + grp) * kBigM4;
  // the four rows of the CTA one residency wave later follow this CTA's
  // (CTA b holds elements [b, b + 1) x kRows4 x kBigM4 of the scratch)
  if (g.ahead && blockIdx.x + g.ahead < gridDim.x)
    prefetch_l2(scratch + (size_t)(blockIdx.x + g.ahead) * (kRows4 * kBigM4), kRows4 * kBigM4 * sizeof(float2), tid,
                kRows4 * TG);
  // every group runs the same passes, so the plan's CTA barriers hold for all four
  ct_local_fft<(int)kBigM4, (int)TG>(s + (size_t)grp * kRowPad4, SampleLoader{row, kBigM4, nullptr}, tw_local,
                                     tid - grp * TG);
  for (uint32_t e = tid; e < kRows4 * kBigM4; e += kRows4 * TG) {
    const uint32_t k2 = e / kRows4, q = e - k2 * kRows4;
    store_bin(out, out_mode, scale, g, beam, r0 + q + g.C * k2, s[(size_t)q * kRowPad4 + sw(k2)]);
  }
}

bool big_size(uint32_t nfft) { return nfft == (1u << 19) || nfft == (1u << 20) || nfft == (1u << 21); }

// Geometry of the row FFTs (M points, C = Cb as the output stride) and the
// W_N table; called by get_plan for big sizes.
spx_status build_big_plan(spx_ctx* ctx, uint32_t nfft, FftPlan* plan) {
  const uint32_t M = big_rows(nfft);
  FftGeom gl{};
  if (!build_geom(M, &gl, kEPTDefault)) return fail(ctx, SPX_ERR_INVALID_ARG, "big plan");
  gl.nfft = nfft;
  gl.C = nfft / M;
  plan->g = gl;
  plan->big = true;
  std::vector<float2> twl(M);
  fill_local_twiddles(gl, twl.data());
  // W_N^{n2 k1} for k1 = a + 16 b as two factor tables, [a][n2] = W_N^{n2 a}
  // (a < 16) and [16 + b][n2] = W_N^{16 n2 b} (b < Cb / 16), then the Cb
  // entries W_Cb^e = W_N^{e M}
  const uint32_t cb = gl.C, J = 16, G = cb / J;
  std::vector<float2> twn((size_t)(J + G) * M + cb);
  auto w_n = [nfft](uint64_t m) {
    m %= nfft;
    const double a = -2.0 * M_PI * (double)m / (double)nfft;
    return make_float2((float)std::cos(a), (float)std::sin(a));
  };
  for (uint32_t a = 0; a < J; ++a)
    for (uint32_t n2 = 0; n2 < M; ++n2) twn[(size_t)a * M + n2] = w_n((uint64_t)n2 * a);
  for (uint32_t b = 0; b < G; ++b)
    for (uint32_t n2 = 0; n2 < M; ++n2) twn[(size_t)(J + b) * M + n2] = w_n((uint64_t)n2 * J * b);
  for (uint32_t e = 0; e < cb; ++e) twn[(size_t)(J + G) * M + e] = w_n((uint64_t)e * M);
  cudaError_t e = cudaMalloc(&plan->d_tw_local, twl.size() * sizeof(float2));
  if (e == cudaSuccess) e = cudaMemcpy(plan->d_tw_local, twl.data(), twl.size() * sizeof(float2), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMalloc(&plan->d_tw_cross, twn.size() * sizeof(float2));
  if (e == cudaSuccess) e = cudaMemcpy(plan->d_tw_cross, twn.data(), twn.size() * sizeof(float2), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "big plan tables");
  return SPX_OK;
}

spx_status launch_fft_big(spx_ctx* ctx, const FftPlan& plan, const float2* d_in, uint32_t beams,
                          uint32_t n_point, const float* d_win, uint32_t out_mode, float scale,
                          void* d_out) {
  if (beams == 0) return SPX_OK;
  const FftGeom& g = plan.g;
  void* scr = nullptr;
  spx_status st = get_scratch(ctx, kSlotExchange, (size_t)beams * g.nfft * sizeof(float2), &scr);
  if (st != SPX_OK) return st;
  float2* scratch = static_cast<float2*>(scr);
  const uint32_t M = g.M;
  // Cb = 128 (2^19 as 128 x 4096, 2^21 as 128 x 16384: 8 x 16) or 256 (2^20
  // as 256 x 4096: 16 x 16, 512 threads, two 16-point stages)
  const uint32_t cthreads = g.C == 256 ? 512u : 256u;
  cudaError_t e = cudaSuccess;
  if (g.C == 128 && M == kBigM4 && !ctx->input_on_host) {
    // 2^19, samples in device memory: the pipelined column kernel (96 KiB,
    // two 256-thread CTAs per SM).
    // Measured against big_cols_kernel (back-to-back calls, same bits):
    // 128 x 2^19 0.505 -> 0.480 ms; for 2^20 (192 KiB, one 512-thread CTA per
    // SM) 0.591 -> 0.615 ms and for 2^21 0.692 -> 0.696 ms, so those keep
    // big_cols_kernel.
    const void* kfn = (const void*)big_cols_pipe_kernel<128, 8>;
    const size_t smem = 3 * (size_t)g.C * 32 * sizeof(float2);  // landing tile + two exchange tiles
    e = configure_kernel(kfn, smem);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "configure big_cols_pipe_kernel");
    const uint32_t tpb = M / 32, total = tpb * beams;
    const uint32_t resident = resident_ctas(kfn, cthreads, smem, 1);
    if (resident == 0) return fail(ctx, SPX_ERR_CUDA, "big_cols_pipe_kernel: no resident CTA");
    const uint32_t ctas = std::min(total, resident);
    void* args[] = {(void*)&d_in,    (void*)&n_point, (void*)&d_win, (void*)&plan.d_tw_cross, (void*)&g.nfft,
                    (void*)&scratch, (void*)&M,       (void*)&tpb,   (void*)&total};
    e = cudaLaunchKernel(kfn, dim3(ctas), dim3(cthreads), args, smem, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "launch big_cols_pipe_kernel");
  } else {
    const void* kcols =
        g.C == 256 ? (const void*)big_cols_kernel<256, 16> : (const void*)big_cols_kernel<128, 8>;
    const size_t csmem = (size_t)g.C * 32 * sizeof(float2);
    e = configure_kernel(kcols, csmem);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "configure big_cols_kernel");
    const uint32_t ahead_cols = ctx->input_on_host ? 0u : resident_ctas(kcols, cthreads, csmem, 1);
    void* cargs[] = {(void*)&d_in, (void*)&n_point, (void*)&d_win, (void*)&plan.d_tw_cross, (void*)&g.nfft,
                     (void*)&scratch, (void*)&ahead_cols, (void*)&M};
    e = cudaLaunchKernel(kcols, dim3(M / 32, beams), dim3(cthreads), cargs, csmem, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "launch big_cols_kernel");
  }
  if (M == kBigM4) {  // four rows per CTA, bin order written directly
    const void* kfn = (const void*)big_rows4_kernel;
    const size_t smem = (size_t)kRows4 * kRowPad4 * sizeof(float2);
    e = configure_kernel(kfn, smem);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "configure big_rows4_kernel");
    FftGeom gg = g;
    gg.beams = beams;
    gg.ahead = ctx->input_on_host ? 0u : resident_ctas(kfn, kRows4 * 256, smem, 1);
    const float2* twl = plan.d_tw_local;
    const float2* scr_c = scratch;
    void* args[] = {(void*)&gg, (void*)&twl, (void*)&scr_c, (void*)&d_out, (void*)&out_mode, (void*)&scale};
    e = cudaLaunchKernel(kfn, dim3(beams * (g.C / kRows4)), dim3(kRows4 * 256), args, smem, ctx->stream);
    return e == cudaSuccess ? SPX_OK : cuda_fail(ctx, e, "launch big_rows4_kernel");
  }
  const void* kfn = (const void*)big_rows_kernel<kEPTDefault>;
  e = configure_kernel(kfn, kMaxFftSmem);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "configure big_rows_kernel");
  FftGeom gg = g;
  gg.beams = beams;
  gg.ahead = resident_ctas(kfn, g.T, (size_t)g.Mpad * sizeof(float2), 1);
  const float2* twl = plan.d_tw_local;
  void* args[] = {(void*)&gg, (void*)&twl, (void*)&scratch};
  e = cudaLaunchKernel(kfn, dim3(beams * g.C), dim3(g.T), args, (size_t)g.Mpad * sizeof(float2), ctx->stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "launch big_rows_kernel");
  return launch_rows_transpose(ctx, g, scratch, beams, d_out, out_mode, scale);
}

}  // namespace spx
