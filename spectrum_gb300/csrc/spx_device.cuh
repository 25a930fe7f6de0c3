// spx_device.cuh — device helpers shared by the FFT and peak kernels.
//
// Complex arithmetic on float2, register-resident forward DFTs of radix
// 2/3/4/6/8/9/16 (natural order in and out), the shared-memory layout used
// by the Stockham passes, and the magnitude formula every kernel uses.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#define SPX_DEV __device__ __forceinline__

namespace spx {

// ---- bounded waits ------------------------------------------------------------
constexpr uint64_t kSpinLimitNs = 1000000000ull;  // 1 s bound on any device-side wait

SPX_DEV uint64_t globaltimer_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// ---- complex helpers -------------------------------------------------------
SPX_DEV float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
SPX_DEV float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
SPX_DEV float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
// a * w (FMA contraction allowed: this is FFT arithmetic, not a parity field)
SPX_DEV float2 cmul(float2 a, float2 w) {
  return make_float2(fmaf(a.x, w.x, -a.y * w.y), fmaf(a.x, w.y, a.y * w.x));
}
SPX_DEV float2 mul_neg_i(float2 a) { return make_float2(a.y, -a.x); }  // a * (-i)
SPX_DEV float2 mul_pos_i(float2 a) { return make_float2(-a.y, a.x); }  // a * (+i)

// |z| and |z|^2 with every operation rounded separately (no FMA contraction),
// i.e. sqrt_rn(re*re + im*im) exactly as a CPU evaluates it in FP32.  Peak
// parity (indices, counts, refined fields) depends on this being the same
// bits in every kernel and in the oracle.
SPX_DEV float mag2_rn(float2 z) { return __fadd_rn(__fmul_rn(z.x, z.x), __fmul_rn(z.y, z.y)); }
SPX_DEV float mag_rn(float2 z) { return __fsqrt_rn(mag2_rn(z)); }

// ---- shared-memory layout ------------------------------------------------------
// Complex element i of a local FFT lives at sw(i) = i + floor(i / 16): one
// unused element after every 16.  A half-warp's 64-bit accesses then hit 16
// different bank pairs for unit strides (every pass's loads), for the stride-R
// stores of a first Stockham pass (R = 2, 4, 8, 16) and for the stores of the
// passes with a stride of 4 or 8.  For d a multiple of 16,
// sw(i + d) = sw(i) + sw(d): strides that are multiples of 16 become constant
// offsets, whatever the local size (power of two or 2^a 3^b).
SPX_DEV uint32_t sw(uint32_t i) { return i + (i >> 4); }
// Shared-memory elements of an n-point local FFT (n rounded up to 16).
constexpr uint32_t sw_len(uint32_t n) { return ((n + 15u) & ~15u) + (((n + 15u) & ~15u) >> 4); }

// ---- constants ---------------------------------------------------------------
constexpr float kS2 = 0.70710678118654752440f;   // sqrt(1/2)
constexpr float kC16 = 0.92387953251128675613f;  // cos(pi/8)
constexpr float kS16 = 0.38268343236508977173f;  // sin(pi/8)
constexpr float kS3 = 0.86602540378443864676f;   // sin(pi/3)
constexpr float kC9a = 0.76604444311897803520f;  // cos(2pi/9)
constexpr float kS9a = 0.64278760968653932632f;  // sin(2pi/9)
constexpr float kC9b = 0.17364817766693034885f;  // cos(4pi/9)
constexpr float kS9b = 0.98480775301220805936f;  // sin(4pi/9)
constexpr float kC9c = 0.93969262078590838405f;  // cos(pi/9)
constexpr float kS9c = 0.34202014332566873304f;  // sin(pi/9)

// ---- forward DFTs in registers (X[k] = sum_n x[n] exp(-2 pi i n k / R)) ----
SPX_DEV void dft2(float2& a, float2& b) {
  float2 t = a;
  a = cadd(t, b);
  b = csub(t, b);
}

SPX_DEV void dft3(float2& a0, float2& a1, float2& a2) {
  float2 t = cadd(a1, a2);
  float2 u = csub(a1, a2);
  float2 m = make_float2(fmaf(-0.5f, t.x, a0.x), fmaf(-0.5f, t.y, a0.y));
  float2 s = cscale(u, kS3);
  a0 = cadd(a0, t);
  a1 = make_float2(m.x + s.y, m.y - s.x);  // m - i*s
  a2 = make_float2(m.x - s.y, m.y + s.x);  // m + i*s
}

SPX_DEV void dft4(float2& a0, float2& a1, float2& a2, float2& a3) {
  float2 s02 = cadd(a0, a2), d02 = csub(a0, a2);
  float2 s13 = cadd(a1, a3), d13 = csub(a1, a3);
  a0 = cadd(s02, s13);
  a2 = csub(s02, s13);
  a1 = make_float2(d02.x + d13.y, d02.y - d13.x);  // d02 - i*d13
  a3 = make_float2(d02.x - d13.y, d02.y + d13.x);  // d02 + i*d13
}

template <int R>
struct Dft;

template <>
struct Dft<2> {
  static SPX_DEV void run(float2* v) { dft2(v[0], v[1]); }
};
template <>
struct Dft<3> {
  static SPX_DEV void run(float2* v) { dft3(v[0], v[1], v[2]); }
};
template <>
struct Dft<4> {
  static SPX_DEV void run(float2* v) { dft4(v[0], v[1], v[2], v[3]); }
};

// 6 = 3 x 2 (Good-Thomas free: twiddles W6^{n2 k1}, n = 2 n1 + n2).
template <>
struct Dft<6> {
  static SPX_DEV void run(float2* v) {
    // n = 2*n1 + n2 (n1 in 0..2, n2 in 0..1); k = k1 + 3*k2
    float2 e0 = v[0], e1 = v[2], e2 = v[4];  // n2 = 0
    float2 o0 = v[1], o1 = v[3], o2 = v[5];  // n2 = 1
    dft3(e0, e1, e2);
    dft3(o0, o1, o2);
    // twiddle W6^{k1} on the n2 = 1 branch: W6^1 = 1/2 - i sqrt(3)/2, W6^2 = -1/2 - i sqrt(3)/2
    o1 = cmul(o1, make_float2(0.5f, -kS3));
    o2 = cmul(o2, make_float2(-0.5f, -kS3));
    v[0] = cadd(e0, o0);
    v[3] = csub(e0, o0);
    v[1] = cadd(e1, o1);
    v[4] = csub(e1, o1);
    v[2] = cadd(e2, o2);
    v[5] = csub(e2, o2);
  }
};

template <>
struct Dft<8> {
  static SPX_DEV void run(float2* v) {
    float2 e0 = v[0], e1 = v[2], e2 = v[4], e3 = v[6];
    float2 o0 = v[1], o1 = v[3], o2 = v[5], o3 = v[7];
    dft4(e0, e1, e2, e3);
    dft4(o0, o1, o2, o3);
    // o1 *= (1 - i)/sqrt2, o2 *= -i, o3 *= (-1 - i)/sqrt2
    o1 = make_float2((o1.x + o1.y) * kS2, (o1.y - o1.x) * kS2);
    o2 = mul_neg_i(o2);
    o3 = make_float2((o3.y - o3.x) * kS2, -(o3.x + o3.y) * kS2);
    v[0] = cadd(e0, o0);
    v[4] = csub(e0, o0);
    v[1] = cadd(e1, o1);
    v[5] = csub(e1, o1);
    v[2] = cadd(e2, o2);
    v[6] = csub(e2, o2);
    v[3] = cadd(e3, o3);
    v[7] = csub(e3, o3);
  }
};

// 9 = 3 x 3: n = 3*n1 + n2, k = k1 + 3*k2, twiddles W9^{n2 k1}.
template <>
struct Dft<9> {
  static SPX_DEV void run(float2* v) {
    float2 b[3][3];
#pragma unroll
    for (int n2 = 0; n2 < 3; ++n2) {
      b[n2][0] = v[n2];
      b[n2][1] = v[3 + n2];
      b[n2][2] = v[6 + n2];
      dft3(b[n2][0], b[n2][1], b[n2][2]);
    }
    // W9^1, W9^2 (n2 = 1: k1 = 1,2), W9^2, W9^4 (n2 = 2: k1 = 1,2)
    b[1][1] = cmul(b[1][1], make_float2(kC9a, -kS9a));
    b[1][2] = cmul(b[1][2], make_float2(kC9b, -kS9b));
    b[2][1] = cmul(b[2][1], make_float2(kC9b, -kS9b));
    b[2][2] = cmul(b[2][2], make_float2(-kC9c, -kS9c));  // W9^4 = cos(8pi/9) - i sin(8pi/9)
#pragma unroll
    for (int k1 = 0; k1 < 3; ++k1) {
      float2 a0 = b[0][k1], a1 = b[1][k1], a2 = b[2][k1];
      dft3(a0, a1, a2);
      v[k1] = a0;
      v[k1 + 3] = a1;
      v[k1 + 6] = a2;
    }
  }
};

// 12 = 3 x 4: n = 4*n1 + n2 (n1 < 3, n2 < 4), k = k1 + 3*k2, twiddles W12^{n2 k1}.
template <>
struct Dft<12> {
  static SPX_DEV void run(float2* v) {
    float2 b[4][3];
#pragma unroll
    for (int n2 = 0; n2 < 4; ++n2) {
      b[n2][0] = v[n2];
      b[n2][1] = v[4 + n2];
      b[n2][2] = v[8 + n2];
      dft3(b[n2][0], b[n2][1], b[n2][2]);
    }
    b[1][1] = cmul(b[1][1], make_float2(kS3, -0.5f));   // W12^1
    b[1][2] = cmul(b[1][2], make_float2(0.5f, -kS3));   // W12^2
    b[2][1] = cmul(b[2][1], make_float2(0.5f, -kS3));   // W12^2
    b[2][2] = cmul(b[2][2], make_float2(-0.5f, -kS3));  // W12^4
    b[3][1] = mul_neg_i(b[3][1]);                        // W12^3
    b[3][2] = make_float2(-b[3][2].x, -b[3][2].y);       // W12^6
#pragma unroll
    for (int k1 = 0; k1 < 3; ++k1) {
      float2 a0 = b[0][k1], a1 = b[1][k1], a2 = b[2][k1], a3 = b[3][k1];
      dft4(a0, a1, a2, a3);
      v[k1] = a0;
      v[k1 + 3] = a1;
      v[k1 + 6] = a2;
      v[k1 + 9] = a3;
    }
  }
};

// 16 = 4 x 4: n = 4*n1 + n2, k = k1 + 4*k2, twiddles W16^{n2 k1}.
template <>
struct Dft<16> {
  static SPX_DEV void run(float2* v) {
    float2 b[4][4];
#pragma unroll
    for (int n2 = 0; n2 < 4; ++n2) {
      b[n2][0] = v[n2];
      b[n2][1] = v[4 + n2];
      b[n2][2] = v[8 + n2];
      b[n2][3] = v[12 + n2];
      dft4(b[n2][0], b[n2][1], b[n2][2], b[n2][3]);
    }
    // n2 = 1: W16^1, W16^2, W16^3
    b[1][1] = cmul(b[1][1], make_float2(kC16, -kS16));
    b[1][2] = make_float2((b[1][2].x + b[1][2].y) * kS2, (b[1][2].y - b[1][2].x) * kS2);
    b[1][3] = cmul(b[1][3], make_float2(kS16, -kC16));
    // n2 = 2: W16^2, W16^4 = -i, W16^6
    b[2][1] = make_float2((b[2][1].x + b[2][1].y) * kS2, (b[2][1].y - b[2][1].x) * kS2);
    b[2][2] = mul_neg_i(b[2][2]);
    b[2][3] = make_float2((b[2][3].y - b[2][3].x) * kS2, -(b[2][3].x + b[2][3].y) * kS2);
    // n2 = 3: W16^3, W16^6, W16^9
    b[3][1] = cmul(b[3][1], make_float2(kS16, -kC16));
    b[3][2] = make_float2((b[3][2].y - b[3][2].x) * kS2, -(b[3][2].x + b[3][2].y) * kS2);
    b[3][3] = cmul(b[3][3], make_float2(-kC16, kS16));
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1) {
      float2 a0 = b[0][k1], a1 = b[1][k1], a2 = b[2][k1], a3 = b[3][k1];
      dft4(a0, a1, a2, a3);
      v[k1] = a0;
      v[k1 + 4] = a1;
      v[k1 + 8] = a2;
      v[k1 + 12] = a3;
    }
  }
};

// ---- top-K lists ------------------------------------------------------------
// A warp's list: lane l holds entry l of its K largest keys (descending; 0 =
// empty).  Inserting key x keeps the K largest.
SPX_DEV uint64_t warp_list_insert(uint64_t mine, uint64_t x, uint32_t lane) {
  const uint64_t up = __shfl_up_sync(0xffffffffu, mine, 1);
  if (mine >= x) return mine;
  return (lane == 0 || up >= x) ? x : up;
}

// Merges the lists of the CTA's nw warps into warp 0's, pairwise in
// log2(nw) rounds (round s: warp w, a multiple of 2s, takes the list of warp
// w + s): K log2(nw) insertions on the critical path instead of K (nw - 1).
// The top K of a union does not depend on the order of the merges, so the
// result is the serial merge's.  lists: nw x 32 words of shared memory, free
// on entry; every thread of the CTA calls it; warp 0 gets the merged entry.
SPX_DEV uint64_t merge_warp_lists(uint64_t* lists, uint64_t mine, uint32_t nw, uint32_t K, uint32_t warp,
                                  uint32_t lane) {
  lists[warp * 32 + lane] = mine;
  for (uint32_t step = 1; step < nw; step *= 2) {
    __syncthreads();
    if (warp % (2 * step) == 0 && warp + step < nw) {
      for (uint32_t e = 0; e < K; ++e) {
        const uint64_t x = lists[(warp + step) * 32 + e];
        if (x == 0) break;
        mine = warp_list_insert(mine, x, lane);
      }
      lists[warp * 32 + lane] = mine;
    }
  }
  return mine;
}

// ---- MaxValue (32 bytes, the reference's GPU layout) -------------------------
struct MaxValueDev {
  uint32_t index;
  float real, imag, magnitude, phase, freq_offset, refined_frequency;
  uint32_t pad;
};

// Radians -> degrees with the reference's constant (fft_kernel_sources_rocm.hpp:247).
constexpr float kRadToDeg = 57.29577951f;

}  // namespace spx
