// fft_big.cu — transforms of 2^19, 2^20 and 2^21 points (the precision
// workload's 2^20-point beams; 2^21 = the reference's nextPow2(2^20) x
// repeat_count 2), beyond what one cluster holds on chip.
//
// nfft = Cb * M with M = 16384 and Cb in {32, 64, 128}; n = M*n1 + n2, k = k1 + Cb*k2:
//   launch 1 (big_cols_kernel): for each n2, the Cb-point DFT over n1 of the
//     windowed, zero-padded samples, times W_N^{n2 k1}, written to
//     scratch[beam][k1][n2] (device memory);
//   launch 2 (big_rows_kernel): for each (beam, k1), the M-point Stockham FFT
//     of row k1 (the passes of fft_core.cuh), X[k1 + Cb*k2] written back over
//     the row it read (scratch[beam][k1][k2], one coalesced pass);
//   launch 3 (rows_transpose_kernel, fft_kernels.cu): scratch[beam][k1][k2]
//     -> bin k1 + Cb*k2 of the output in the requested mode, written in
//     contiguous runs (written straight from launch 2, the stride-Cb stores
//     kept its SMs waiting on the store queue: 0.63 ms for 64 x 2^20 points).
// All twiddles are FP64-generated and stored in FP32 (W_N^{n2 k1} in a table
// of nfft entries laid out [k1][n2], so a warp's 32 columns read 256
// contiguous bytes; W_M from the local plan), which is what the 120 dB
// dynamic range of the precision workload needs.  Replaces hipFFT's internal
// multi-pass plan for large sizes (src/fft_func/src/fft_processor_rocm.cpp:176-193).
#include <cmath>
#include <vector>

#include "fft_core.cuh"
#include "spx_internal.h"

namespace spx {

constexpr uint32_t kBigM = 16384;

// One tile = 32 consecutive n2 columns x Cb rows (n1); lane = column, warp
// t = row group (tile reads conflict-free, output rows written 256 bytes at a time).
template <int CB>
__global__ void __launch_bounds__(256)
big_cols_kernel(const float2* __restrict__ in, uint32_t n_point, const float* __restrict__ win,
                const float2* __restrict__ twN, uint32_t nfft, float2* __restrict__ scratch,
                uint32_t ahead) {
  __shared__ float2 tile[CB][33];
  const uint32_t tid = threadIdx.x;
  const uint32_t beam = blockIdx.y, n2_0 = blockIdx.x * 32;
  const float2* x = in + (size_t)beam * n_point;
  {  // L2 prefetch of the 32-column tile of the CTA `ahead` places later
    const uint64_t f = (uint64_t)blockIdx.y * gridDim.x + blockIdx.x + ahead;
    if (ahead && f < (uint64_t)gridDim.x * gridDim.y && tid < CB) {
      const uint32_t fb = (uint32_t)(f / gridDim.x), fc = (uint32_t)(f % gridDim.x) * 32;
      const uint32_t lo = tid * kBigM + fc, hi = min(lo + 32, n_point);
      if (lo < hi) prefetch_l2(in + (size_t)fb * n_point + lo, (size_t)(hi - lo) * sizeof(float2), 0, 1);
    }
  }
  for (uint32_t e = tid; e < CB * 32; e += 256) {
    const uint32_t n1 = e >> 5, col = e & 31;
    tile[n1][col] = load_sample(x, n1 * kBigM + n2_0 + col, n_point, win);
  }
  __syncthreads();
  const uint32_t col = tid & 31, t = tid >> 5;
  constexpr int J = CB / 8;  // stage-1 radix (4, 8 or 16)
  // stage 1: thread t transforms rows t + 8j (j < J), twiddles W_CB^{t a}
  float2 v[J];
#pragma unroll
  for (int j = 0; j < J; ++j) v[j] = tile[t + 8 * j][col];
  Dft<J>::run(v);
#pragma unroll
  for (int a = 1; a < J; ++a) {
    const uint32_t e = (t * a) % CB;
    v[a] = cmul(v[a], __ldg(twN + nfft + e));  // W_CB^e, after the [k1][n2] table
  }
  __syncthreads();
#pragma unroll
  for (int a = 0; a < J; ++a) tile[t + 8 * a][col] = v[a];
  __syncthreads();
  // stage 2: for a = t, t + 8, ... (< J), the 8-point DFT over t' of rows t' + 8a -> k1 = a + J*b
#pragma unroll
  for (uint32_t a = t; a < (uint32_t)J; a += 8) {
    float2 w[8];
#pragma unroll
    for (int tp = 0; tp < 8; ++tp) w[tp] = tile[tp + 8 * a][col];
    Dft<8>::run(w);
    const uint32_t n2 = n2_0 + col;
    float2* o = scratch + (size_t)beam * nfft + n2;
#pragma unroll
    for (int b = 0; b < 8; ++b) {
      const uint32_t k1 = a + J * b;
      o[(size_t)k1 * kBigM] = cmul(w[b], __ldg(twN + (size_t)k1 * kBigM + n2));  // W_N^{n2 k1}
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

bool big_size(uint32_t nfft) { return nfft == (1u << 19) || nfft == (1u << 20) || nfft == (1u << 21); }

// Geometry of the row FFTs (M = 16384, C = Cb as the output stride) and the
// W_N table; called by get_plan for big sizes.
spx_status build_big_plan(spx_ctx* ctx, uint32_t nfft, FftPlan* plan) {
  FftGeom gl{};
  if (!build_geom(kBigM, &gl, kEPTDefault)) return fail(ctx, SPX_ERR_INVALID_ARG, "big plan");
  gl.nfft = nfft;
  gl.C = nfft / kBigM;
  plan->g = gl;
  plan->big = true;
  std::vector<float2> twl(kBigM);
  fill_local_twiddles(gl, twl.data());
  // [k1][n2] = W_N^{n2 k1} (n2 < kBigM, k1 < Cb, so n2 k1 < nfft: no reduction),
  // then the Cb entries W_Cb^e = W_N^{e kBigM}
  const uint32_t cb = gl.C;
  std::vector<float2> twn((size_t)nfft + cb);
  auto w_n = [nfft](uint64_t m) {
    const double a = -2.0 * M_PI * (double)m / (double)nfft;
    return make_float2((float)std::cos(a), (float)std::sin(a));
  };
  for (uint32_t k1 = 0; k1 < cb; ++k1)
    for (uint32_t n2 = 0; n2 < kBigM; ++n2) twn[(size_t)k1 * kBigM + n2] = w_n((uint64_t)n2 * k1);
  for (uint32_t e = 0; e < cb; ++e) twn[(size_t)nfft + e] = w_n((uint64_t)e * kBigM);
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
  dim3 grid(kBigM / 32, beams);
  const void* kcols = g.C == 128 ? (const void*)big_cols_kernel<128>
                      : g.C == 64 ? (const void*)big_cols_kernel<64> : (const void*)big_cols_kernel<32>;
  const uint32_t ahead_cols = ctx->input_on_host ? 0u : resident_ctas(kcols, 256, 0, 1);
  if (g.C == 128)
    big_cols_kernel<128><<<grid, 256, 0, ctx->stream>>>(d_in, n_point, d_win, plan.d_tw_cross, g.nfft, scratch,
                                                        ahead_cols);
  else if (g.C == 64)
    big_cols_kernel<64><<<grid, 256, 0, ctx->stream>>>(d_in, n_point, d_win, plan.d_tw_cross, g.nfft, scratch,
                                                       ahead_cols);
  else
    big_cols_kernel<32><<<grid, 256, 0, ctx->stream>>>(d_in, n_point, d_win, plan.d_tw_cross, g.nfft, scratch,
                                                       ahead_cols);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(ctx, e, "launch big_cols_kernel");
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
