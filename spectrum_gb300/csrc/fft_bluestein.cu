// fft_bluestein.cu — transforms of any length without a direct plan (not
// 2^a 3^b, e.g. 1000 = 2^3 5^3 or a prime), up to 2^27 points.
//
// The reference's CpuFFT takes any length (pocketfft,
// include/spectrum/utils/cpu_fft.hpp:68-89); this is the GPU counterpart for
// the lengths the Stockham plans do not cover.  Bluestein's chirp-z identity
// n k = (n^2 + k^2 - (k - n)^2) / 2 turns the N-point DFT into a circular
// convolution of length m >= 2N - 1 (a power of two, m <= 2^28):
//   w[n] = exp(-i pi n^2 / N)
//   X[k] = w[k] * sum_n (x[n] w[n]) conj(w[k - n])
//        = w[k] * IFFT_m( FFT_m(a) * FFT_m(b) )[k],
//   a[n] = x[n] w[n] (n < N, 0 up to m), b[j] = conj(w[j]) at j and m - j.
// Four launches per call: the pre-multiplied, zero-padded sequence, the
// m-point transform (the library's own plan), the product with FFT_m(b) (made
// once per plan on the device), the m-point inverse transform (the forward
// plan with the reversing 1/m epilogue of spx_ifft), and the post-multiply
// with the output epilogue of spx_fft (any output mode).  w is FP64-generated
// (n^2 reduced mod 2N exactly in integers) and stored FP32.  Error: a few
// FP32 transforms of m points, ~1e-6 of the peak.
#include <cmath>
#include <vector>

#include "fft_core.cuh"
#include "spx_internal.h"

namespace spx {

bool bluestein_size(uint32_t nfft) {
  FftGeom g;
  return nfft >= 2 && nfft <= kMaxBluestein && !build_geom(nfft, &g) && !big_size(nfft) && !huge_size(nfft);
}

static uint32_t bluestein_m(uint32_t nfft) {
  uint32_t m = 1;
  while (m < 2 * nfft - 1) m <<= 1;
  return m;
}

// a[beam][n] = x[n] win[n] w[n] for n < n_point, 0 for n_point <= n < m.
__global__ void chirp_pre_kernel(const float2* __restrict__ x, uint32_t n_point, const float* __restrict__ win,
                                 const float2* __restrict__ w, uint32_t m, uint64_t total,
                                 float2* __restrict__ a) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t beam = i / m;
    const uint32_t n = (uint32_t)(i - beam * m);
    float2 v = make_float2(0.f, 0.f);
    if (n < n_point) v = cmul(load_sample(x + beam * n_point, n, n_point, win), __ldg(w + n));
    a[i] = v;
  }
}

// A[beam][k] *= B[k].
__global__ void chirp_mul_kernel(float2* __restrict__ A, const float2* __restrict__ B, uint32_t m, uint64_t total) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (uint64_t)gridDim.x * blockDim.x)
    A[i] = cmul(A[i], __ldg(B + (i % m)));
}

// X[k] = w[k] c[beam][k] for k < N, in output mode out_mode (store_bin).
__global__ void chirp_post_kernel(const float2* __restrict__ c, const float2* __restrict__ w, FftGeom g, uint32_t m,
                                  uint64_t total, void* __restrict__ out, uint32_t out_mode, float scale) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t beam = (uint32_t)(i / g.nfft);
    const uint32_t k = (uint32_t)(i - (uint64_t)beam * g.nfft);
    store_bin(out, out_mode, scale, g, beam, k, cmul(c[(size_t)beam * m + k], __ldg(w + k)));
  }
}

static unsigned grid_for(uint64_t total, int sms) {
  const uint64_t want = (total + 255) / 256;
  return (unsigned)std::min<uint64_t>(want, (uint64_t)sms * 8);
}

spx_status build_bluestein_plan(spx_ctx* ctx, uint32_t nfft, FftPlan* plan) {
  const uint32_t m = bluestein_m(nfft);
  const FftPlan* sub = nullptr;
  spx_status st = get_plan(ctx, m, &sub);
  if (st != SPX_OK) return st;
  plan->bluestein = true;
  plan->bm = m;
  plan->sub = sub;
  plan->g = FftGeom{};
  plan->g.nfft = nfft;
  // w[n] = exp(-i pi n^2 / N): n^2 mod 2N exactly, then the angle in FP64
  std::vector<float2> w(nfft), b((size_t)m, make_float2(0.f, 0.f));
  for (uint32_t n = 0; n < nfft; ++n) {
    const uint64_t r = ((uint64_t)n * n) % (2ull * nfft);
    const double a = -M_PI * (double)r / (double)nfft;
    w[n] = make_float2((float)std::cos(a), (float)std::sin(a));
    const float2 cw = make_float2(w[n].x, -w[n].y);
    b[n] = cw;
    if (n > 0) b[m - n] = cw;
  }
  cudaError_t e = cudaMalloc(&plan->d_chirp, (size_t)nfft * sizeof(float2));
  if (e == cudaSuccess) e = cudaMalloc(&plan->d_bfft, (size_t)m * sizeof(float2));
  if (e == cudaSuccess)
    e = cudaMemcpy(plan->d_chirp, w.data(), (size_t)nfft * sizeof(float2), cudaMemcpyHostToDevice);
  // FFT_m(b), once, by the library's own m-point transform (b staged in d_bfft, transformed in place)
  if (e == cudaSuccess) e = cudaMemcpy(plan->d_bfft, b.data(), (size_t)m * sizeof(float2), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "Bluestein plan tables");
  st = launch_fft_out(ctx, *sub, plan->d_bfft, 1, m, nullptr, SPX_OUT_COMPLEX, 1.0f, plan->d_bfft);
  if (st != SPX_OK) return st;
  e = cudaStreamSynchronize(ctx->stream);
  return e == cudaSuccess ? SPX_OK : cuda_fail(ctx, e, "Bluestein plan");
}

spx_status launch_fft_bluestein(spx_ctx* ctx, const FftPlan& plan, const float2* d_in, uint32_t beams,
                                uint32_t n_point, const float* d_win, uint32_t out_mode, float scale,
                                void* d_out) {
  if (beams == 0) return SPX_OK;
  const uint32_t m = plan.bm, N = plan.g.nfft;
  void* buf = nullptr;
  spx_status st = get_scratch(ctx, kSlotChirp, (size_t)beams * m * sizeof(float2), &buf);
  if (st != SPX_OK) return st;
  float2* a = static_cast<float2*>(buf);
  const uint64_t tm = (uint64_t)beams * m;
  chirp_pre_kernel<<<grid_for(tm, ctx->sm_count), 256, 0, ctx->stream>>>(d_in, n_point, d_win, plan.d_chirp, m, tm, a);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(ctx, e, "launch chirp_pre_kernel");
  st = launch_fft_out(ctx, *plan.sub, a, beams, m, nullptr, SPX_OUT_COMPLEX, 1.0f, a);
  if (st != SPX_OK) return st;
  chirp_mul_kernel<<<grid_for(tm, ctx->sm_count), 256, 0, ctx->stream>>>(a, plan.d_bfft, m, tm);
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(ctx, e, "launch chirp_mul_kernel");
  st = launch_fft_out(ctx, *plan.sub, a, beams, m, nullptr, kOutComplexReversed, 1.0f / (float)m, a);
  if (st != SPX_OK) return st;
  const uint64_t tn = (uint64_t)beams * N;
  chirp_post_kernel<<<grid_for(tn, ctx->sm_count), 256, 0, ctx->stream>>>(a, plan.d_chirp, plan.g, m, tn, d_out,
                                                                            out_mode, scale);
  e = cudaGetLastError();
  return e == cudaSuccess ? SPX_OK : cuda_fail(ctx, e, "launch chirp_post_kernel");
}

}  // namespace spx
