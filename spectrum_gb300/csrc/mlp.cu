// mlp.cu — learned sub-bin refinement of spectral peaks.
//
// No reference counterpart: the reference refines a peak with a 3-point
// parabola on |X| (include/spectrum/kernels/fft_kernel_sources_rocm.hpp:228-239),
// which for a Hann window is biased by up to a few hundredths of a bin
// (scalloping).  Here a small network learns the offset and the amplitude
// correction from the 5 bins around the peak.
//
// Network: 10 -> 64 -> 64 -> 2, GELU (erf form) after both hidden layers.
//   input : |X[k+d]| / |X[k]|                                   d = -2..2
//           wrap(arg(X[k+d] conj X[k]) + pi d (n_point-1)/nfft)  d = -2..2
//           (the linear phase of a symmetric window starting at sample 0 is
//            removed, so main-lobe phases sit near 0 and do not wrap)
//   output: y0 = offset of the tone from bin k, in bins
//           y1 = log(tone amplitude / |X[k]|)
// Weights: FP32 masters (Adam) and a BF16 copy; every product reads the BF16
// weights and accumulates in FP32; biases stay FP32.
// Training data comes from the library's own FFT: single-tone frames, features
// from the frame's nfft-point Hann spectrum, labels from a 16x zero-padded FFT
// of the same windowed frame (peak on the fine grid + 3-point parabola there).
// Inference keeps the parabolic result whenever the network's offset leaves
// the bin (|y0| > 0.5) or is not finite.
//
// Parameter layout (floats): W1[64][10] b1[64] W2[64][64] b2[64] W3[2][64] b3[2].
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <new>
#include <vector>

#include "mlp_device.cuh"
#include "spx_device.cuh"
#include "spx_internal.h"

namespace spx {

SPX_DEV float gelu_grad(float z) {
  return 0.5f * (1.0f + erff(z * 0.70710678118654752f)) +
         z * 0.39894228040143268f * expf(-0.5f * z * z);
}

// ---- training layers (one thread per output element) ---------------------------
// Z[b][o] = sum_i X[b][i] W[o][i] + bias[o];  H = GELU(Z) when act, else Z.
__global__ void mlp_fwd_kernel(const float* __restrict__ X, const __nv_bfloat16* __restrict__ W,
                               const float* __restrict__ bias, uint32_t B, int in, int out,
                               float* __restrict__ Z, float* __restrict__ H, int act) {
  const uint64_t idx = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (uint64_t)B * out) return;
  const uint32_t b = idx / out, o = idx % out;
  const float* x = X + (size_t)b * in;
  const __nv_bfloat16* w = W + (size_t)o * in;
  float acc = bias[o];
  for (int i = 0; i < in; ++i) acc = fmaf(x[i], __bfloat162float(w[i]), acc);
  Z[idx] = acc;
  if (H) H[idx] = act ? gelu(acc) : acc;
}

// Mean squared error over the rows with mask != 0 (mask may be null):
// dY = (Y - T) * 2 / (B * kOut) on those rows, 0 elsewhere; loss += MSE.
__global__ void mlp_out_grad_kernel(const float* __restrict__ Y, const float* __restrict__ Tg,
                                    const uint32_t* __restrict__ mask, uint32_t B,
                                    float* __restrict__ dY, float* __restrict__ loss) {
  const uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x;
  float l = 0.f;
  if (idx < B * kOut) {
    const bool on = !mask || mask[idx / kOut] != 0;
    const float d = on ? Y[idx] - Tg[idx] : 0.f;
    dY[idx] = d * (2.0f / (float)(B * kOut));
    l = d * d / (float)(B * kOut);
  }
  for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
  if (loss && (threadIdx.x & 31) == 0) atomicAdd(loss, l);
}

// dX[b][i] = (sum_o dZ[b][o] W[o][i]) * GELU'(Zprev[b][i])
__global__ void mlp_bwd_data_kernel(const float* __restrict__ dZ, const __nv_bfloat16* __restrict__ W,
                                    const float* __restrict__ Zprev, uint32_t B, int in, int out,
                                    float* __restrict__ dX) {
  const uint64_t idx = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (uint64_t)B * in) return;
  const uint32_t b = idx / in, i = idx % in;
  const float* dz = dZ + (size_t)b * out;
  float acc = 0.f;
  for (int o = 0; o < out; ++o) acc = fmaf(dz[o], __bfloat162float(W[(size_t)o * in + i]), acc);
  dX[idx] = acc * gelu_grad(Zprev[idx]);
}

// Partial weight gradients of one chunk of kBwdChunk rows (blockIdx.y):
// part[chunk][o*in + i] = sum_b dZ[b][o] X[b][i] and part[chunk][out*in + o]
// = sum_b dZ[b][o] over the chunk's rows b, in row order.  mlp_sum_chunks
// then adds the chunks in chunk order: the gradient is the same bits on every
// run (no atomics), so training is reproducible.
constexpr uint32_t kBwdChunk = 512;
constexpr uint32_t kMaxLayerParams = kH * (kH + 1);  // largest out * (in + 1)
__global__ void mlp_bwd_weight_kernel(const float* __restrict__ dZ, const float* __restrict__ X,
                                      uint32_t B, int in, int out, float* __restrict__ part) {
  const uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t n = (uint32_t)(out * (in + 1));
  if (idx >= n) return;
  const uint32_t o = idx / (in + 1), i = idx % (in + 1);
  const uint32_t b0 = blockIdx.y * kBwdChunk, b1 = min(B, b0 + kBwdChunk);
  float acc = 0.f;
  float* dst = part + (size_t)blockIdx.y * n;
  if (i < (uint32_t)in) {
    for (uint32_t b = b0; b < b1; ++b) acc = fmaf(dZ[(size_t)b * out + o], X[(size_t)b * in + i], acc);
    dst[o * in + i] = acc;
  } else {
    for (uint32_t b = b0; b < b1; ++b) acc += dZ[(size_t)b * out + o];
    dst[out * in + o] = acc;
  }
}

// g[idx] = sum over chunks c = 0, 1, ... of part[c][idx] (a layer's W then b,
// contiguous in the parameter layout).
__global__ void mlp_sum_chunks_kernel(const float* __restrict__ part, uint32_t chunks, uint32_t n,
                                      float* __restrict__ g) {
  const uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= n) return;
  float acc = 0.f;
  for (uint32_t c = 0; c < chunks; ++c) acc += part[(size_t)c * n + idx];
  g[idx] = acc;
}

// Adam on the FP32 masters (bias-corrected), then the BF16 copy.
__global__ void mlp_adam_kernel(float* __restrict__ p, float* __restrict__ m, float* __restrict__ v,
                                const float* __restrict__ g, __nv_bfloat16* __restrict__ pb,
                                uint32_t n, float lr, float b1, float b2, float eps, float c1,
                                float c2) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  const float pi = p[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  p[i] = pi;
  pb[i] = __float2bfloat16_rn(pi);
}

__global__ void to_bf16_kernel(const float* __restrict__ p, __nv_bfloat16* __restrict__ pb, uint32_t n) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) pb[i] = __float2bfloat16_rn(p[i]);
}

// Row gather for one minibatch: row j of the batch is training row
// (a * (first + j) + c) mod n — an affine permutation of [0, n) (a odd, n a
// power of two) that changes every epoch.
__global__ void mlp_gather_kernel(const float* __restrict__ feat, const float* __restrict__ tgt,
                                  const uint32_t* __restrict__ valid, uint32_t n, uint32_t first,
                                  uint32_t B, uint32_t a, uint32_t c, float* __restrict__ bx,
                                  float* __restrict__ bt, uint32_t* __restrict__ bm) {
  const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= B) return;
  const uint32_t r = (a * (first + j) + c) & (n - 1);
  for (int i = 0; i < kIn; ++i) bx[(size_t)j * kIn + i] = feat[(size_t)r * kIn + i];
  bt[(size_t)j * 2] = tgt[(size_t)r * 2];
  bt[(size_t)j * 2 + 1] = tgt[(size_t)r * 2 + 1];
  bm[j] = valid ? valid[r] : 1u;
}

// ---- features -------------------------------------------------------------------
// Features of the peak at bin k of a spectrum in device memory (needs bins
// k-2..k+2); false at the edges or when |X[k]| is 0.
struct GlobalBins {
  const float2* f;
  SPX_DEV float2 operator()(uint32_t k) const { return f[k]; }
};
SPX_DEV bool peak_features(const float2* f, uint32_t n_point, uint32_t nfft, uint32_t k, float* feat) {
  return peak_features_at(GlobalBins{f}, n_point, nfft, k, feat);
}

// ---- training data ----------------------------------------------------------------
SPX_DEV uint64_t mix64(uint64_t z) {  // splitmix64 finaliser
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
SPX_DEV float u01(uint64_t key) { return (float)(mix64(key) >> 40) * (1.0f / 16777216.0f); }
SPX_DEV float gauss(uint64_t key) {  // Box-Muller, one of the pair
  const float u1 = fmaxf(u01(key), 1e-7f), u2 = u01(key ^ 0xA5A5A5A5A5A5A5A5ull);
  return sqrtf(-2.f * logf(u1)) * cospif(2.f * u2);
}

// One single-tone frame per block: x[t] = exp(i(2 pi f t + phi)) + sigma (n_re + i n_im),
// f ~ U[fmin, fmax) cycles/sample, phi ~ U[0, 2 pi), SNR ~ U[snr_lo, snr_hi] dB
// (sigma = 10^(-SNR/20), total complex noise power sigma^2).
__global__ void gen_frames_kernel(uint64_t seed, uint32_t frame0, uint32_t n, float fmin,
                                  float fmax, float snr_lo, float snr_hi, float2* __restrict__ x,
                                  float* __restrict__ truth) {
  const uint32_t fr = blockIdx.x;
  const uint64_t key = mix64(seed ^ mix64(frame0 + fr));
  const float f = fmin + (fmax - fmin) * u01(key ^ 1);
  const float ph = u01(key ^ 2);  // cycles
  const float snr = snr_lo + (snr_hi - snr_lo) * u01(key ^ 3);
  const float s = powf(10.f, -snr / 20.f) * 0.70710678118654752f;
  if (threadIdx.x == 0 && truth) {
    truth[(size_t)fr * 2] = f;
    truth[(size_t)fr * 2 + 1] = snr;
  }
  for (uint32_t t = threadIdx.x; t < n; t += blockDim.x) {
    const double cyc = (double)f * (double)t + (double)ph;
    const float frac = (float)(cyc - floor(cyc));
    float sn, cs;
    sincospif(2.f * frac, &sn, &cs);
    const uint64_t nk = mix64(key + t);
    x[(size_t)fr * n + t] = make_float2(cs + s * gauss(nk), sn + s * gauss(nk ^ 0x5851F42D4C957F2Dull));
  }
}

// Per frame: k = argmax |X| over [2, nfft/2 - 2) (largest value, lowest bin);
// features at k; labels from the 16x zero-padded spectrum X16 (fine-grid peak
// within +-24 fine bins of 16 k, then a 3-point parabola on the fine grid):
// target = (fine offset, log(fine amplitude / |X[k]|)); parabolic = (k, the
// 3-point coarse parabola offset: the method without the network); valid = 0
// for unusable frames.
__global__ void frame_labels_kernel(const float2* __restrict__ X, const float2* __restrict__ X16,
                                    uint32_t nfft, float* __restrict__ feat, float* __restrict__ tgt,
                                    float* __restrict__ par, uint32_t* __restrict__ valid) {
  const uint32_t fr = blockIdx.x;
  const float2* f = X + (size_t)fr * nfft;
  const float2* g = X16 + (size_t)fr * nfft * 16;
  __shared__ uint64_t best[32];
  uint64_t key = 0;
  for (uint32_t k = 2 + threadIdx.x; k + 2 < nfft / 2; k += blockDim.x) {
    const uint64_t kk = ((uint64_t)__float_as_uint(mag_rn(f[k])) << 32) | (uint32_t)(~k);
    key = kk > key ? kk : key;
  }
  for (int o = 16; o > 0; o >>= 1) {
    const uint64_t w = __shfl_xor_sync(0xffffffffu, key, o);
    key = w > key ? w : key;
  }
  if ((threadIdx.x & 31) == 0) best[threadIdx.x >> 5] = key;
  __syncthreads();
  if (threadIdx.x != 0) return;
  for (uint32_t w = 1; w < blockDim.x / 32; ++w) key = best[w] > key ? best[w] : key;
  const uint32_t k = ~(uint32_t)key;
  float fe[kIn];
  bool ok = key != 0 && peak_features(f, nfft, nfft, k, fe);
  float off = 0.f, la = 0.f, pd = 0.f;
  if (ok) {
    uint32_t mbest = 16 * k;
    float vbest = -1.f;
    for (int d = -24; d <= 24; ++d) {
      const uint32_t m = 16 * k + d;
      const float v = mag_rn(g[m]);
      if (v > vbest) { vbest = v; mbest = m; }
    }
    const float yl = mag_rn(g[mbest - 1]), yc = vbest, yr = mag_rn(g[mbest + 1]);
    const float den = yl - 2.f * yc + yr;
    const float dfine = fabsf(den) > 1e-20f ? fminf(fmaxf(0.5f * (yl - yr) / den, -0.5f), 0.5f) : 0.f;
    const float amp = yc - 0.25f * (yl - yr) * dfine;
    const float mc = mag_rn(f[k]);
    off = ((float)mbest - 16.f * (float)k + dfine) * (1.f / 16.f);
    la = logf(amp / mc);
    ok = amp > 0.f && fabsf(off) < 1.0f && isfinite(la);
    const float cl = mag_rn(f[k - 1]), cr = mag_rn(f[k + 1]);
    const float cden = cl - 2.f * mc + cr;
    pd = fabsf(cden) > 1e-10f ? fminf(fmaxf(0.5f * (cl - cr) / cden, -0.5f), 0.5f) : 0.f;
  }
  for (int i = 0; i < kIn; ++i) feat[(size_t)fr * kIn + i] = ok ? fe[i] : 0.f;
  tgt[(size_t)fr * 2] = ok ? off : 0.f;
  tgt[(size_t)fr * 2 + 1] = ok ? la : 0.f;
  par[(size_t)fr * 2] = (float)k;
  par[(size_t)fr * 2 + 1] = pd;
  valid[fr] = ok ? 1u : 0u;
}

// ---- inference: one warp per peak ------------------------------------------------
// mlp_forward_warp (mlp_device.cuh): lane l owns hidden units l and l + 32 of
// both layers; the layer-1 outputs go through a per-warp shared row; the 2
// outputs are warp sums.  Weights are staged once per block in shared memory
// (BF16 values widened to FP32, exact).
constexpr int kRefineWarps = 8;
struct RefineSmem {
  MlpWeights w;
  float h[kRefineWarps][kH];
  float x[kRefineWarps][kIn];
};

__global__ void __launch_bounds__(kRefineWarps * 32)
mlp_refine_kernel(const __nv_bfloat16* __restrict__ pb, const float* __restrict__ p,
                  const float2* __restrict__ fft, uint32_t n_point, uint32_t nfft, uint32_t beams,
                  uint32_t K, float fs, MaxValueDev* __restrict__ peaks,
                  const uint32_t* __restrict__ counts, float* __restrict__ amp_out,
                  uint32_t* __restrict__ used_mlp) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  RefineSmem& s = *reinterpret_cast<RefineSmem*>(smem_raw);
  mlp_stage(s.w, pb, p, threadIdx.x, blockDim.x);
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint64_t total = (uint64_t)beams * K;
  const uint64_t stride = (uint64_t)gridDim.x * kRefineWarps;
  for (uint64_t idx = (uint64_t)blockIdx.x * kRefineWarps + warp; idx < total; idx += stride) {
    const uint32_t beam = (uint32_t)(idx / K), j = (uint32_t)(idx % K);
    if (j >= counts[beam]) continue;  // warp-uniform
    MaxValueDev mv = peaks[idx];
    // the features, offset d = lane - 2 on lanes 0..4 (peak_features_at's
    // arithmetic, one offset per lane)
    const uint32_t k = mv.index;
    const GlobalBins bins{fft + (size_t)beam * nfft};
    bool good = k >= 2 && k + 2 < nfft;
    float2 c = make_float2(0.f, 0.f);
    float mc = 0.f;
    if (good) {
      c = bins(k);
      mc = mag_rn(c);
      good = mc > 0.f;
    }
    if (good && lane < 5)
      peak_feature_pair(bins, c, mc, peak_lin(n_point, nfft), k, (int)lane - 2, &s.x[warp][lane], &s.x[warp][lane + 5]);
    __syncwarp();
    float y0 = 0.f, y1 = 0.f;
    if (good) mlp_forward_warp(s.w, s.x[warp], s.h[warp], lane, &y0, &y1);
    __syncwarp();
    if (lane == 0) {
      float amp;
      const bool use = mlp_apply(mv, good, y0, y1, fs, nfft, &amp);
      if (use) peaks[idx] = mv;
      if (amp_out) amp_out[idx] = amp;
      if (used_mlp) used_mlp[idx] = use ? 1u : 0u;
    }
  }
}

}  // namespace spx

// ---------------------------------------------------------------------------
// Host
// ---------------------------------------------------------------------------
using namespace spx;

struct spx_mlp {
  int device = 0;
  float* d_p = nullptr;           // FP32 masters
  float* d_m = nullptr;           // Adam first moment
  float* d_v = nullptr;           // Adam second moment
  float* d_g = nullptr;           // gradients
  __nv_bfloat16* d_pb = nullptr;  // BF16 copy read by every product
  float* d_work = nullptr;        // activations and minibatch rows
  size_t work_floats = 0;
  uint64_t step = 0;              // Adam step count
};

namespace spx {
void mlp_device_params(const spx_mlp* mlp, const void** pb, const float** p, int* device) {
  *pb = mlp->d_pb;
  *p = mlp->d_p;
  *device = mlp->device;
}
}  // namespace spx

namespace {

unsigned nblocks(uint64_t n, unsigned t) { return (unsigned)((n + t - 1) / t); }

// Per row: Z1 H1 Z2 H2 (4 x 64), Y (2), dZ2 dZ1 (2 x 64), dY (2), then the
// minibatch slot: x (10), t (2), mask (1 word).
constexpr size_t kWorkPerRow = 4 * kH + kOut + 2 * kH + kOut + kIn + 2 + 1;

struct Acts {
  float *Z1, *H1, *Z2, *H2, *Y, *dZ2, *dZ1, *dY, *bx, *bt;
  uint32_t* bm;
  float* part;  // per-chunk partial weight gradients, ceil(B / kBwdChunk) x kMaxLayerParams
};

spx_status ensure_work(spx_ctx* ctx, spx_mlp* m, uint32_t B, Acts* a) {
  const size_t chunks = (B + kBwdChunk - 1) / kBwdChunk;
  const size_t need = (size_t)B * kWorkPerRow + chunks * kMaxLayerParams;
  if (m->work_floats < need) {
    cudaError_t e = cudaSuccess;
    if (m->d_work) e = cudaStreamSynchronize(ctx->stream);
    if (e == cudaSuccess && m->d_work) e = cudaFree(m->d_work);
    m->d_work = nullptr;
    m->work_floats = 0;
    if (e == cudaSuccess) e = cudaMalloc(&m->d_work, need * sizeof(float));
    if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaMalloc(mlp activations)");
    m->work_floats = need;
  }
  float* w = m->d_work;
  a->Z1 = w;
  a->H1 = a->Z1 + (size_t)B * kH;
  a->Z2 = a->H1 + (size_t)B * kH;
  a->H2 = a->Z2 + (size_t)B * kH;
  a->Y = a->H2 + (size_t)B * kH;
  a->dZ2 = a->Y + (size_t)B * kOut;
  a->dZ1 = a->dZ2 + (size_t)B * kH;
  a->dY = a->dZ1 + (size_t)B * kH;
  a->bx = a->dY + (size_t)B * kOut;
  a->bt = a->bx + (size_t)B * kIn;
  a->bm = reinterpret_cast<uint32_t*>(a->bt + (size_t)B * 2);
  a->part = w + (size_t)B * kWorkPerRow;
  return SPX_OK;
}

void forward(spx_ctx* ctx, spx_mlp* m, const float* X, uint32_t B, const Acts& a) {
  const float* p = m->d_p;
  const __nv_bfloat16* pb = m->d_pb;
  cudaStream_t s = ctx->stream;
  mlp_fwd_kernel<<<nblocks((uint64_t)B * kH, 256), 256, 0, s>>>(X, pb + kOffW1, p + kOffB1, B, kIn, kH, a.Z1, a.H1, 1);
  mlp_fwd_kernel<<<nblocks((uint64_t)B * kH, 256), 256, 0, s>>>(a.H1, pb + kOffW2, p + kOffB2, B, kH, kH, a.Z2, a.H2, 1);
  mlp_fwd_kernel<<<nblocks((uint64_t)B * kOut, 256), 256, 0, s>>>(a.H2, pb + kOffW3, p + kOffB3, B, kH, kOut, a.Y, nullptr, 0);
}

// Weight and bias gradients of one layer (in -> out) into g (W then b),
// through per-chunk partial sums added in a fixed order.
void layer_weight_grad(cudaStream_t s, const float* dZ, const float* X, uint32_t B, int in, int out,
                       const Acts& a, float* g) {
  const unsigned ch = (B + kBwdChunk - 1) / kBwdChunk;
  const uint32_t n = (uint32_t)(out * (in + 1));
  mlp_bwd_weight_kernel<<<dim3(nblocks(n, 128), ch), 128, 0, s>>>(dZ, X, B, in, out, a.part);
  mlp_sum_chunks_kernel<<<nblocks(n, 128), 128, 0, s>>>(a.part, ch, n, g);
}

// Gradient of the masked MSE into m->d_g (every entry written, the same bits
// on every run); loss accumulated into d_loss.
void backward(spx_ctx* ctx, spx_mlp* m, const float* X, const float* Tg, const uint32_t* mask,
              uint32_t B, const Acts& a, float* d_loss) {
  cudaStream_t s = ctx->stream;
  const __nv_bfloat16* pb = m->d_pb;
  float* g = m->d_g;
  mlp_out_grad_kernel<<<nblocks((uint64_t)B * kOut, 256), 256, 0, s>>>(a.Y, Tg, mask, B, a.dY, d_loss);
  layer_weight_grad(s, a.dY, a.H2, B, kH, kOut, a, g + kOffW3);
  mlp_bwd_data_kernel<<<nblocks((uint64_t)B * kH, 256), 256, 0, s>>>(a.dY, pb + kOffW3, a.Z2, B, kH, kOut, a.dZ2);
  layer_weight_grad(s, a.dZ2, a.H1, B, kH, kH, a, g + kOffW2);
  mlp_bwd_data_kernel<<<nblocks((uint64_t)B * kH, 256), 256, 0, s>>>(a.dZ2, pb + kOffW2, a.Z1, B, kH, kH, a.dZ1);
  layer_weight_grad(s, a.dZ1, X, B, kIn, kH, a, g + kOffW1);
}

void adam(spx_ctx* ctx, spx_mlp* m, float lr) {
  m->step += 1;
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.f - (float)std::pow(0.9, (double)m->step);
  const float c2 = 1.f - (float)std::pow(0.999, (double)m->step);
  mlp_adam_kernel<<<nblocks(kNParams, 256), 256, 0, ctx->stream>>>(m->d_p, m->d_m, m->d_v, m->d_g, m->d_pb,
                                                                   kNParams, lr, b1, b2, 1e-8f, c1, c2);
}

spx_status launch_status(spx_ctx* ctx, const char* what) {
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? SPX_OK : cuda_fail(ctx, e, what);
}

}  // namespace

extern "C" {

uint32_t spx_mlp_param_count(void) { return kNParams; }

spx_status spx_mlp_create(spx_ctx* ctx, uint64_t seed, spx_mlp** out) {
  if (!ctx || !out) return SPX_ERR_INVALID_ARG;
  *out = nullptr;
  DeviceGuard guard(ctx->device);
  auto* m = new (std::nothrow) spx_mlp();
  if (!m) return fail(ctx, SPX_ERR_OUT_OF_MEMORY, "spx_mlp_create: host allocation failed");
  m->device = ctx->device;
  cudaError_t e = cudaSuccess;
  float** bufs[] = {&m->d_p, &m->d_m, &m->d_v, &m->d_g};
  for (float** b : bufs)
    if (e == cudaSuccess) e = cudaMalloc(b, kNParams * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&m->d_pb, kNParams * sizeof(__nv_bfloat16));
  if (e != cudaSuccess) {
    spx_mlp_destroy(m);
    return cuda_fail(ctx, e, "cudaMalloc(mlp parameters)");
  }
  // Uniform (He-style) initialisation from a seeded 64-bit LCG; biases 0.
  std::vector<float> p(kNParams, 0.f);
  uint64_t st = seed;
  auto next = [&]() {
    st = st * 6364136223846793005ull + 1442695040888963407ull;
    return (double)(st >> 11) * (2.0 / 9007199254740992.0) - 1.0;  // U[-1, 1)
  };
  for (int i = 0; i < kH * kIn; ++i) p[kOffW1 + i] = (float)(next() * std::sqrt(6.0 / kIn));
  for (int i = 0; i < kH * kH; ++i) p[kOffW2 + i] = (float)(next() * std::sqrt(6.0 / kH));
  for (int i = 0; i < kOut * kH; ++i) p[kOffW3 + i] = (float)(next() * std::sqrt(1.0 / kH));
  const spx_status s = spx_mlp_set_params(ctx, m, p.data());
  if (s != SPX_OK) {
    spx_mlp_destroy(m);
    return s;
  }
  *out = m;
  return SPX_OK;
}

spx_status spx_mlp_destroy(spx_mlp* m) {
  if (!m) return SPX_OK;
  DeviceGuard guard(m->device);
  cudaFree(m->d_p);
  cudaFree(m->d_m);
  cudaFree(m->d_v);
  cudaFree(m->d_g);
  cudaFree(m->d_pb);
  cudaFree(m->d_work);
  delete m;
  return SPX_OK;
}

spx_status spx_mlp_set_params(spx_ctx* ctx, spx_mlp* m, const float* host_params) {
  if (!ctx || !m || !host_params) return SPX_ERR_INVALID_ARG;
  DeviceGuard guard(ctx->device);
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  if (e == cudaSuccess) e = cudaMemcpy(m->d_p, host_params, kNParams * sizeof(float), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(m->d_m, 0, kNParams * sizeof(float));
  if (e == cudaSuccess) e = cudaMemset(m->d_v, 0, kNParams * sizeof(float));
  if (e != cudaSuccess) return cuda_fail(ctx, e, "spx_mlp_set_params");
  to_bf16_kernel<<<nblocks(kNParams, 256), 256, 0, ctx->stream>>>(m->d_p, m->d_pb, kNParams);
  m->step = 0;
  e = cudaStreamSynchronize(ctx->stream);
  return e == cudaSuccess ? SPX_OK : cuda_fail(ctx, e, "spx_mlp_set_params");
}

spx_status spx_mlp_get_params(spx_ctx* ctx, spx_mlp* m, float* host_params) {
  if (!ctx || !m || !host_params) return SPX_ERR_INVALID_ARG;
  DeviceGuard guard(ctx->device);
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  if (e == cudaSuccess) e = cudaMemcpy(host_params, m->d_p, kNParams * sizeof(float), cudaMemcpyDeviceToHost);
  return e == cudaSuccess ? SPX_OK : cuda_fail(ctx, e, "spx_mlp_get_params");
}

spx_status spx_mlp_forward(spx_ctx* ctx, spx_mlp* m, const float* d_x, uint32_t rows, float* d_y) {
  if (!ctx || !m) return SPX_ERR_INVALID_ARG;
  if (rows == 0) return SPX_OK;
  if (!d_x || !d_y) return fail(ctx, SPX_ERR_INVALID_ARG, "spx_mlp_forward: null pointer");
  DeviceGuard guard(ctx->device);
  Acts a;
  spx_status st = ensure_work(ctx, m, rows, &a);
  if (st != SPX_OK) return st;
  forward(ctx, m, d_x, rows, a);
  cudaMemcpyAsync(d_y, a.Y, (size_t)rows * kOut * sizeof(float), cudaMemcpyDeviceToDevice, ctx->stream);
  return launch_status(ctx, "spx_mlp_forward");
}

spx_status spx_mlp_gradients(spx_ctx* ctx, spx_mlp* m, const float* d_x, const float* d_t,
                             const uint32_t* d_mask, uint32_t rows, float* d_grad, float* d_loss) {
  if (!ctx || !m) return SPX_ERR_INVALID_ARG;
  if (!d_x || !d_t || !d_grad || rows == 0)
    return fail(ctx, SPX_ERR_INVALID_ARG, "spx_mlp_gradients: null pointer or no rows");
  DeviceGuard guard(ctx->device);
  Acts a;
  spx_status st = ensure_work(ctx, m, rows, &a);
  if (st != SPX_OK) return st;
  forward(ctx, m, d_x, rows, a);
  backward(ctx, m, d_x, d_t, d_mask, rows, a, d_loss);
  cudaMemcpyAsync(d_grad, m->d_g, kNParams * sizeof(float), cudaMemcpyDeviceToDevice, ctx->stream);
  return launch_status(ctx, "spx_mlp_gradients");
}

spx_status spx_mlp_train_step(spx_ctx* ctx, spx_mlp* m, const float* d_x, const float* d_t,
                              const uint32_t* d_mask, uint32_t rows, float lr, float* d_loss) {
  if (!ctx || !m) return SPX_ERR_INVALID_ARG;
  if (!d_x || !d_t || rows == 0)
    return fail(ctx, SPX_ERR_INVALID_ARG, "spx_mlp_train_step: null pointer or no rows");
  if (!(lr > 0.f) || !std::isfinite(lr)) return fail(ctx, SPX_ERR_INVALID_ARG, "spx_mlp_train_step: lr must be > 0");
  DeviceGuard guard(ctx->device);
  Acts a;
  spx_status st = ensure_work(ctx, m, rows, &a);
  if (st != SPX_OK) return st;
  forward(ctx, m, d_x, rows, a);
  backward(ctx, m, d_x, d_t, d_mask, rows, a, d_loss);
  adam(ctx, m, lr);
  return launch_status(ctx, "spx_mlp_train_step");
}

spx_status spx_mlp_train(spx_ctx* ctx, spx_mlp* m, const float* d_feat, const float* d_target,
                         const uint32_t* d_valid, uint32_t rows, uint32_t batch, uint32_t epochs,
                         float lr_max, float lr_min, uint64_t seed, float* d_epoch_loss) {
  if (!ctx || !m) return SPX_ERR_INVALID_ARG;
  if (!d_feat || !d_target) return fail(ctx, SPX_ERR_INVALID_ARG, "spx_mlp_train: null pointer");
  if (rows == 0 || (rows & (rows - 1)) || batch == 0 || batch > rows)
    return fail(ctx, SPX_ERR_INVALID_ARG, "spx_mlp_train: rows must be a power of two >= batch > 0");
  if (!(lr_max > 0.f) || !(lr_min > 0.f) || lr_min > lr_max || !std::isfinite(lr_max))
    return fail(ctx, SPX_ERR_INVALID_ARG, "spx_mlp_train: need 0 < lr_min <= lr_max");
  DeviceGuard guard(ctx->device);
  Acts a;
  spx_status st = ensure_work(ctx, m, batch, &a);
  if (st != SPX_OK) return st;
  if (d_epoch_loss) cudaMemsetAsync(d_epoch_loss, 0, (size_t)epochs * sizeof(float), ctx->stream);
  const uint32_t steps_per_epoch = rows / batch;
  const double total = (double)steps_per_epoch * epochs;
  uint64_t rs = seed;
  auto next = [&]() {
    rs = rs * 6364136223846793005ull + 1442695040888963407ull;
    return (uint32_t)(rs >> 32);
  };
  uint64_t step = 0;
  for (uint32_t ep = 0; ep < epochs; ++ep) {
    const uint32_t pa = next() | 1u, pc = next();
    for (uint32_t s = 0; s < steps_per_epoch; ++s, ++step) {
      // cosine decay from lr_max to lr_min over the whole run
      const double cosv = 0.5 * (1.0 + std::cos(3.14159265358979323846 * (double)step / total));
      const float lr = (float)(lr_min + (lr_max - lr_min) * cosv);
      mlp_gather_kernel<<<nblocks(batch, 256), 256, 0, ctx->stream>>>(d_feat, d_target, d_valid, rows,
                                                                      s * batch, batch, pa, pc, a.bx, a.bt, a.bm);
      forward(ctx, m, a.bx, batch, a);
      backward(ctx, m, a.bx, a.bt, a.bm, batch, a, d_epoch_loss ? d_epoch_loss + ep : nullptr);
      adam(ctx, m, lr);
    }
    st = launch_status(ctx, "spx_mlp_train");
    if (st != SPX_OK) return st;
  }
  // per-epoch loss: mean over the epoch's steps
  if (d_epoch_loss) {
    std::vector<float> h(epochs);
    cudaError_t e = cudaMemcpyAsync(h.data(), d_epoch_loss, epochs * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    for (auto& v : h) v /= (float)steps_per_epoch;
    if (e == cudaSuccess) e = cudaMemcpy(d_epoch_loss, h.data(), epochs * sizeof(float), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "spx_mlp_train loss");
  }
  return SPX_OK;
}

spx_status spx_mlp_make_frames(spx_ctx* ctx, uint64_t seed, uint32_t frame0, uint32_t frames,
                               uint32_t nfft, float snr_lo_db, float snr_hi_db, float* d_feat,
                               float* d_target, float* d_parabolic, uint32_t* d_valid,
                               float* d_truth) {
  if (!ctx) return SPX_ERR_INVALID_ARG;
  if (frames == 0) return SPX_OK;
  if (!d_feat || !d_target || !d_parabolic || !d_valid)
    return fail(ctx, SPX_ERR_INVALID_ARG, "spx_mlp_make_frames: null pointer");
  if (nfft < 64 || nfft > 4096 || (nfft & (nfft - 1)))
    return fail(ctx, SPX_ERR_INVALID_ARG, "spx_mlp_make_frames: nfft must be a power of two in [64, 4096]");
  if (!(snr_lo_db <= snr_hi_db) || !std::isfinite(snr_lo_db) || !std::isfinite(snr_hi_db))
    return fail(ctx, SPX_ERR_INVALID_ARG, "spx_mlp_make_frames: need finite snr_lo_db <= snr_hi_db");
  DeviceGuard guard(ctx->device);
  // frames x, spectra X and 16x zero-padded judge spectra X16, chunk by chunk
  const uint32_t chunk = std::min<uint32_t>(frames, (1u << 24) / nfft);
  const size_t pts = (size_t)chunk * nfft;
  void* scr = nullptr;
  spx_status st = get_scratch(ctx, kSlotSpectrum, 18 * pts * sizeof(float2), &scr);
  if (st != SPX_OK) return st;
  float2* x = static_cast<float2*>(scr);
  float2* X = x + pts;
  float2* X16 = X + pts;
  const float fmin = 4.0f / nfft, fmax = 0.5f - 4.0f / nfft;
  for (uint32_t f0 = 0; f0 < frames; f0 += chunk) {
    const uint32_t n = std::min(chunk, frames - f0);
    gen_frames_kernel<<<n, 256, 0, ctx->stream>>>(seed, frame0 + f0, nfft, fmin, fmax, snr_lo_db, snr_hi_db, x,
                                                  d_truth ? d_truth + (size_t)f0 * 2 : nullptr);
    st = launch_status(ctx, "spx_mlp_make_frames");
    if (st != SPX_OK) return st;
    st = spx_fft(ctx, x, n, nfft, nfft, SPX_WINDOW_HANN, SPX_OUT_COMPLEX, 1.0f, X);
    if (st != SPX_OK) return st;
    st = spx_fft(ctx, x, n, nfft, nfft * 16, SPX_WINDOW_HANN, SPX_OUT_COMPLEX, 1.0f, X16);
    if (st != SPX_OK) return st;
    frame_labels_kernel<<<n, 256, 0, ctx->stream>>>(X, X16, nfft, d_feat + (size_t)f0 * kIn,
                                                    d_target + (size_t)f0 * 2, d_parabolic + (size_t)f0 * 2,
                                                    d_valid + f0);
    st = launch_status(ctx, "spx_mlp_make_frames");
    if (st != SPX_OK) return st;
  }
  return SPX_OK;
}

spx_status spx_mlp_refine(spx_ctx* ctx, spx_mlp* m, const void* d_fft, uint32_t beams,
                          uint32_t n_point, uint32_t nfft, float sample_rate, uint32_t K,
                          spx_max_value* d_peaks, const uint32_t* d_counts, float* d_amplitude,
                          uint32_t* d_used_mlp) {
  if (!ctx || !m) return SPX_ERR_INVALID_ARG;
  if ((uint64_t)beams * K == 0) return SPX_OK;
  if (!d_fft || !d_peaks || !d_counts) return fail(ctx, SPX_ERR_INVALID_ARG, "spx_mlp_refine: null pointer");
  if (nfft < 5 || n_point == 0 || n_point > nfft)
    return fail(ctx, SPX_ERR_INVALID_ARG, "spx_mlp_refine: need 5 <= nfft and 0 < n_point <= nfft");
  DeviceGuard guard(ctx->device);
  const size_t smem = sizeof(RefineSmem);
  cudaError_t e = cudaFuncSetAttribute(mlp_refine_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "spx_mlp_refine: configure");
  const uint64_t warps = (uint64_t)beams * K;
  const unsigned grid = (unsigned)std::min<uint64_t>((warps + kRefineWarps - 1) / kRefineWarps,
                                                     (uint64_t)ctx->sm_count * 8);
  mlp_refine_kernel<<<grid, kRefineWarps * 32, smem, ctx->stream>>>(
      m->d_pb, m->d_p, static_cast<const float2*>(d_fft), n_point, nfft, beams, K, sample_rate,
      reinterpret_cast<MaxValueDev*>(d_peaks), d_counts, d_amplitude, d_used_mlp);
  return launch_status(ctx, "spx_mlp_refine");
}

}  // extern "C"
