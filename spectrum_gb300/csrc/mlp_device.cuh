// mlp_device.cuh — the learned refinement of one peak, shared by the
// standalone refine kernel (mlp.cu) and the fused FFT + top-K + refinement
// kernel (fft_peaks.cu), so both give the same bits.
//
// Network: 10 -> 64 -> 64 -> 2, GELU (erf form) after both hidden layers.
//   input : |X[k+d]| / |X[k]|                                   d = -2..2
//           wrap(arg(X[k+d] conj X[k]) + pi d (n_point-1)/nfft)  d = -2..2
//   output: y0 = offset of the tone from bin k, in bins
//           y1 = log(tone amplitude / |X[k]|)
// Parameter layout (floats): W1[64][10] b1[64] W2[64][64] b2[64] W3[2][64] b3[2];
// the products read the BF16 copy of the weights, widened to FP32 (exact).
#pragma once

#include <cuda_bf16.h>

#include "spx_device.cuh"

namespace spx {

constexpr int kIn = 10, kH = 64, kOut = 2;
constexpr int kOffW1 = 0, kOffB1 = kOffW1 + kH * kIn, kOffW2 = kOffB1 + kH,
              kOffB2 = kOffW2 + kH * kH, kOffW3 = kOffB2 + kH, kOffB3 = kOffW3 + kOut * kH,
              kNParams = kOffB3 + kOut;  // 4994
static_assert(kNParams == 4994, "parameter layout");

SPX_DEV float gelu(float z) { return 0.5f * z * (1.0f + erff(z * 0.70710678118654752f)); }

SPX_DEV float wrap_pi(float a) {
  const float tp = 6.28318530717958647692f;
  return a - tp * rintf(a * 0.15915494309189535f);
}

// pi (n_point - 1) / nfft: the window centre's linear phase per bin.
SPX_DEV float peak_lin(uint32_t n_point, uint32_t nfft) {
  return 3.14159265358979324f * (float)(n_point - 1) / (float)nfft;
}

// The two features of offset d (-2..2) of the peak at bin k, whose bin is c
// with |c| = mc > 0: |X[k+d]| / |X[k]| and the wrapped phase of
// X[k+d] conj X[k] plus lin d (0 for d = 0).  Every path computes its
// features through this function, so they have the same bits.
template <typename Bin>
SPX_DEV void peak_feature_pair(const Bin& bin, float2 c, float mc, float lin, uint32_t k, int d, float* ratio,
                               float* phase) {
  const float2 z = bin(k + d);
  *ratio = mag_rn(z) / mc;
  // z * conj(c)
  const float re = fmaf(z.x, c.x, z.y * c.y), im = fmaf(z.y, c.x, -z.x * c.y);
  *phase = d == 0 ? 0.f : wrap_pi(atan2f(im, re) + lin * (float)d);
}

// Features of the peak at bin k (bins k-2..k+2 through bin(k), complex);
// false at the edges or when |X[k]| is 0.
template <typename Bin>
SPX_DEV bool peak_features_at(const Bin& bin, uint32_t n_point, uint32_t nfft, uint32_t k, float* feat) {
  if (k < 2 || k + 2 >= nfft) return false;
  const float2 c = bin(k);
  const float mc = mag_rn(c);
  if (!(mc > 0.f)) return false;
  const float lin = peak_lin(n_point, nfft);
#pragma unroll
  for (int d = -2; d <= 2; ++d) peak_feature_pair(bin, c, mc, lin, k, d, &feat[d + 2], &feat[d + 7]);
  return true;
}

// The weights in shared memory as FP32; the hidden layers' matrices
// transposed to [input][unit] (w1t[i * kH + o] = W1[o][i], likewise w2t), so
// the 32 lanes of a warp, one unit each, read 32 consecutive words: no bank
// conflicts (the parameter layout [unit][input] put every lane of a warp on
// one bank).  The layout does not change any sum's order.
struct MlpWeights {
  float w1t[kIn * kH], b1[kH], w2t[kH * kH], b2[kH], w3[kOut * kH], b3[kOut];
};

// Stages the weights (BF16 products, FP32 biases) by threads tid, tid + n, ...
SPX_DEV void mlp_stage(MlpWeights& w, const __nv_bfloat16* __restrict__ pb, const float* __restrict__ p,
                       uint32_t tid, uint32_t n) {
  for (uint32_t i = tid; i < kH * kIn; i += n) {  // W1[o][c], i = o kIn + c
    const uint32_t o = i / kIn, c = i - o * kIn;
    w.w1t[c * kH + o] = __bfloat162float(pb[kOffW1 + i]);
  }
  for (uint32_t i = tid; i < kH * kH; i += n) {  // W2[o][c], i = o kH + c
    const uint32_t o = i / kH, c = i - o * kH;
    w.w2t[c * kH + o] = __bfloat162float(pb[kOffW2 + i]);
  }
  for (uint32_t i = tid; i < kOut * kH; i += n) w.w3[i] = __bfloat162float(pb[kOffW3 + i]);
  for (uint32_t i = tid; i < kH; i += n) {
    w.b1[i] = p[kOffB1 + i];
    w.b2[i] = p[kOffB2 + i];
  }
  if (tid < kOut) w.b3[tid] = p[kOffB3 + tid];
}

// The network on the features x[kIn] by one warp (lane l owns hidden units
// l and l + 32 of both layers; h: the warp's 64-float row for layer 1's
// outputs; y0, y1 are warp sums, returned to every lane).
SPX_DEV void mlp_forward_warp(const MlpWeights& w, const float* x, float* h, uint32_t lane, float* y0,
                              float* y1) {
  float a0 = w.b1[lane], a1 = w.b1[lane + 32];
#pragma unroll
  for (int i = 0; i < kIn; ++i) {
    const float xi = x[i];
    a0 = fmaf(xi, w.w1t[i * kH + lane], a0);
    a1 = fmaf(xi, w.w1t[i * kH + lane + 32], a1);
  }
  h[lane] = gelu(a0);
  h[lane + 32] = gelu(a1);
  __syncwarp();
  float c0 = w.b2[lane], c1 = w.b2[lane + 32];
#pragma unroll 16
  for (int i = 0; i < kH; ++i) {
    const float hi = h[i];
    c0 = fmaf(hi, w.w2t[i * kH + lane], c0);
    c1 = fmaf(hi, w.w2t[i * kH + lane + 32], c1);
  }
  const float g0 = gelu(c0), g1 = gelu(c1);
  float s0 = fmaf(g0, w.w3[lane], g1 * w.w3[lane + 32]);
  float s1 = fmaf(g0, w.w3[kH + lane], g1 * w.w3[kH + lane + 32]);
  for (int o = 16; o > 0; o >>= 1) {
    s0 += __shfl_xor_sync(0xffffffffu, s0, o);
    s1 += __shfl_xor_sync(0xffffffffu, s1, o);
  }
  *y0 = s0 + w.b3[0];
  *y1 = s1 + w.b3[1];
}

// The refined record: the network's offset replaces the parabolic one unless
// it leaves the bin or is not finite; returns whether it was used and the
// amplitude |X[k]| exp(y1) (|X[k]| when not used).
SPX_DEV bool mlp_apply(MaxValueDev& mv, bool good, float y0, float y1, float fs, uint32_t nfft, float* amp) {
  const bool use = good && isfinite(y0) && isfinite(y1) && fabsf(y0) <= 0.5f;
  if (use) {
    mv.freq_offset = y0;
    mv.refined_frequency = __fmul_rn(__fadd_rn((float)mv.index, y0), __fdiv_rn(fs, (float)nfft));
  }
  *amp = use ? mv.magnitude * expf(y1) : mv.magnitude;
  return use;
}

}  // namespace spx
