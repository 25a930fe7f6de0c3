// fft_huge.cu — transforms of more than 2^21 points: nfft = N1 x N2 with
// N1 and N2 2^a 3^b sizes of at most 16384 points each (every power of two
// from 2^22 to 2^28, and the 3-smooth sizes in that range with such a
// split).  The reference's FFTProcessorROCm::CalculateNFFT takes any
// nextPow2(n_point) x repeat_count (src/fft_func/src/fft_processor_rocm.cpp:673-677)
// and hands it to hipFFT; Bluestein's method (fft_bluestein.cu) runs its
// power-of-two transforms of more than 2^21 points here too.
//
// Four steps with explicit transposes (n = N2 n1 + n2, k = k1 + N1 k2):
//   1. A[n2][n1] = w[n] x[n] (0 for n >= n_point)       huge_transpose_kernel, kIn
//   2. each row A[n2][.] <- FFT_N1, in place             the library's N1-point plan
//   3. B[k1][n2] = A[n2][k1] W_N^{n2 k1}                 huge_transpose_kernel, kTwiddle
//   4. each row B[k1][.] <- FFT_N2, in place             the library's N2-point plan
//   5. X[k1 + N1 k2] = B[k1][k2] in the output mode      huge_transpose_kernel, kOut
// Each transpose moves 32 x 32 tiles through shared memory (pitch 33:
// conflict-free both ways), read and written in 256-byte runs.  The
// twiddle W_N^m (m = n2 k1 < N) is W_N^{(m div L) L} x W_N^{m mod L} from two
// tables of FP64-generated FP32 values (L = 2^ceil(log2(N) / 2)): one complex
// multiply, ~2 ulps.  Steps 2 and 4 are single-CTA transforms (N1, N2 <=
// 16384), so the device memory of a call is two scratch buffers of
// beams x N points (the context's kSlotHuge).
#include <cmath>
#include <vector>

#include "fft_core.cuh"
#include "spx_internal.h"

namespace spx {

constexpr uint32_t kHugeMin = 1u << 22;
constexpr uint32_t kHugeMaxFactor = 16384;

// The split N1 x N2 of nfft (both 2^a 3^b, <= 16384, N1 <= N2, N1 the
// largest such divisor); false when nfft has none.
static bool huge_split(uint32_t nfft, uint32_t* n1, uint32_t* n2) {
  if (nfft < kHugeMin || nfft > kMaxHuge || !is_smooth23(nfft)) return false;
  uint32_t best = 0;
  for (uint64_t p2 = 1; p2 <= kHugeMaxFactor; p2 *= 2)
    for (uint64_t d = p2; d <= kHugeMaxFactor; d *= 3) {
      if (nfft % d) continue;
      const uint64_t e = nfft / d;
      if (d <= e && e <= kHugeMaxFactor && d > best) best = (uint32_t)d;
    }
  if (!best) return false;
  *n1 = best;
  *n2 = nfft / best;
  return true;
}

bool huge_size(uint32_t nfft) {
  uint32_t a, b;
  return huge_split(nfft, &a, &b);
}

enum HugeStep : uint32_t { kIn = 0, kTwiddle = 1, kOut = 2 };

struct HugeArgs {
  uint32_t rows, cols;   // the per-beam matrix read: rows x cols, row-major
  uint32_t n_point;      // kIn: samples per beam
  uint32_t lshift;       // kTwiddle: L = 2^lshift
  const float* win;      // kIn: window table (null: none)
  const float2* lo;      // kTwiddle: W_N^l, l < L
  const float2* hi;      // kTwiddle: W_N^{j L}
  uint32_t out_mode;     // kOut
  float scale;           // kOut
  FftGeom g;             // kOut: nfft for store_bin
};

// One 32 x 32 tile of beam blockIdx.z: element (r, c) of the rows x cols
// matrix `in` goes to element (c, r) of the cols x rows matrix `out`, or,
// for kOut, to bin r + rows * c of the output in its mode.
//   kIn:      in = the samples: element (n1, n2) is sample n = n1 * cols + n2
//             (windowed, 0 beyond n_point);
//   kTwiddle: element (n2, k1) is multiplied by W_N^{n2 k1};
//   kOut:     element (k1, k2) is bin k1 + rows * k2.
template <uint32_t STEP>
__global__ void __launch_bounds__(256)
huge_transpose_kernel(HugeArgs h, const float2* __restrict__ in, void* __restrict__ out) {
  __shared__ float2 tile[32][33];
  const uint32_t tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const uint32_t c0 = blockIdx.x * 32, r0 = blockIdx.y * 32, beam = blockIdx.z;
  const uint64_t per_beam = (uint64_t)h.rows * h.cols;
#pragma unroll
  for (uint32_t j = 0; j < 32; j += 8) {
    const uint32_t r = r0 + ty + j, c = c0 + tx;
    float2 v = make_float2(0.f, 0.f);
    if (r < h.rows && c < h.cols) {
      if constexpr (STEP == kIn) {
        const uint32_t n = r * h.cols + c;  // < nfft <= 2^28
        v = load_sample(in + (size_t)beam * h.n_point, n, h.n_point, h.win);
      } else {
        v = __ldcs(in + beam * per_beam + (size_t)r * h.cols + c);
        if constexpr (STEP == kTwiddle) {
          const uint32_t m = r * c;  // n2 k1 < nfft
          v = cmul(v, cmul(__ldg(h.hi + (m >> h.lshift)), __ldg(h.lo + (m & ((1u << h.lshift) - 1u)))));
        }
      }
    }
    tile[ty + j][tx] = v;
  }
  __syncthreads();
#pragma unroll
  for (uint32_t j = 0; j < 32; j += 8) {
    const uint32_t c = c0 + ty + j, r = r0 + tx;  // write element (r, c) at (c, r)
    if (r < h.rows && c < h.cols) {
      const float2 v = tile[tx][ty + j];
      if constexpr (STEP == kOut)
        store_bin(out, h.out_mode, h.scale, h.g, beam, r + h.rows * c, v);
      else
        __stcg(reinterpret_cast<float2*>(out) + beam * per_beam + (size_t)c * h.rows + r, v);
    }
  }
}

spx_status build_huge_plan(spx_ctx* ctx, uint32_t nfft, FftPlan* plan) {
  uint32_t n1 = 0, n2 = 0;
  if (!huge_split(nfft, &n1, &n2)) return fail(ctx, SPX_ERR_INVALID_ARG, "huge plan: no split");
  const FftPlan* p1 = nullptr;
  const FftPlan* p2 = nullptr;
  spx_status st = get_plan(ctx, n1, &p1);
  if (st == SPX_OK) st = get_plan(ctx, n2, &p2);
  if (st != SPX_OK) return st;
  plan->huge = true;
  plan->hn1 = n1;
  plan->hn2 = n2;
  plan->sub = p1;
  plan->sub2 = p2;
  plan->g = FftGeom{};
  plan->g.nfft = nfft;
  uint32_t lshift = 0;
  while ((1ull << (2 * lshift)) < nfft) ++lshift;  // L = 2^ceil(log2(N) / 2), L^2 >= N
  plan->hlshift = lshift;
  const uint64_t L = 1ull << lshift, H = (nfft + L - 1) / L;
  std::vector<float2> t(L + H);
  auto w = [nfft](uint64_t m) {
    const double a = -2.0 * M_PI * (double)(m % nfft) / (double)nfft;
    return make_float2((float)std::cos(a), (float)std::sin(a));
  };
  for (uint64_t l = 0; l < L; ++l) t[l] = w(l);
  for (uint64_t j = 0; j < H; ++j) t[L + j] = w(j * L);
  cudaError_t e = cudaMalloc(&plan->d_tw_cross, t.size() * sizeof(float2));
  if (e == cudaSuccess) e = cudaMemcpy(plan->d_tw_cross, t.data(), t.size() * sizeof(float2), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "huge plan tables");
  return SPX_OK;
}

spx_status launch_fft_huge(spx_ctx* ctx, const FftPlan& plan, const float2* d_in, uint32_t beams,
                           uint32_t n_point, const float* d_win, uint32_t out_mode, float scale,
                           void* d_out) {
  if (beams == 0) return SPX_OK;
  if (beams > 65535) return fail(ctx, SPX_ERR_INVALID_ARG, "transforms of more than 2^21 points take <= 65535 beams");
  const uint32_t N = plan.g.nfft, n1 = plan.hn1, n2 = plan.hn2;
  const size_t bytes = (size_t)beams * N * sizeof(float2);
  void* buf = nullptr;
  spx_status st = get_scratch(ctx, kSlotHuge, 2 * bytes, &buf);
  if (st != SPX_OK) return st;
  float2* A = static_cast<float2*>(buf);
  float2* B = A + (size_t)beams * N;
  HugeArgs h{};
  h.win = d_win;
  h.n_point = n_point;
  h.lshift = plan.hlshift;
  h.lo = plan.d_tw_cross;
  h.hi = plan.d_tw_cross + (1u << plan.hlshift);
  h.out_mode = out_mode;
  h.scale = scale;
  h.g = plan.g;
  auto grid = [beams](uint32_t rows, uint32_t cols) { return dim3((cols + 31) / 32, (rows + 31) / 32, beams); };
  // 1. samples as N1 rows of N2 -> A: N2 rows of N1
  h.rows = n1;
  h.cols = n2;
  huge_transpose_kernel<kIn><<<grid(n1, n2), 256, 0, ctx->stream>>>(h, d_in, A);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(ctx, e, "launch huge_transpose_kernel (in)");
  // 2. N1-point transforms of the N2 rows of every beam
  st = launch_fft_out(ctx, *plan.sub, A, beams * n2, n1, nullptr, SPX_OUT_COMPLEX, 1.0f, A);
  if (st != SPX_OK) return st;
  // 3. twiddles, A: N2 rows of N1 -> B: N1 rows of N2
  h.rows = n2;
  h.cols = n1;
  huge_transpose_kernel<kTwiddle><<<grid(n2, n1), 256, 0, ctx->stream>>>(h, A, B);
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(ctx, e, "launch huge_transpose_kernel (twiddle)");
  // 4. N2-point transforms of the N1 rows
  st = launch_fft_out(ctx, *plan.sub2, B, beams * n1, n2, nullptr, SPX_OUT_COMPLEX, 1.0f, B);
  if (st != SPX_OK) return st;
  // 5. B: N1 rows (k1) of N2 (k2) -> bin k1 + N1 k2
  h.rows = n1;
  h.cols = n2;
  huge_transpose_kernel<kOut><<<grid(n1, n2), 256, 0, ctx->stream>>>(h, B, d_out);
  e = cudaGetLastError();
  return e == cudaSuccess ? SPX_OK : cuda_fail(ctx, e, "launch huge_transpose_kernel (out)");
}

}  // namespace spx
