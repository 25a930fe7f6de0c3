// fft_core.cuh — the FFT building blocks used by every spectrum kernel.
//
// One beam of nfft = C * M points is transformed by C CTAs (C = 1 for
// nfft <= 16384).  Index maps (n = M*n1 + n2, k = k1 + C*k2):
//
//   X[k1 + C*k2] = sum_{n2} W_M^{n2 k2} * ( W_N^{n2 k1} * sum_{n1} x[M n1 + n2] W_C^{n1 k1} )
//
// * cross stage (C > 1): CTA c takes n2 in its slice of [0, M), reads the C
//   samples x[M n1 + n2] straight from device memory (window and zero
//   padding applied on load), does the C-point DFT in registers, applies
//   W_N^{n2 k1} and writes element k1 to row k1 of its cluster's exchange
//   slot in device memory (L2-resident).
// * local stage: after a cluster barrier CTA k1 runs an M-point Stockham
//   FFT over row k1 (first pass reading device memory, the others in place
//   in shared memory, radix 16/9/8/4/3/2 in registers) and ends with
//   Z[k2] = X[k1 + C*k2] in natural order.
// * C = 1: the first Stockham pass reads the samples from device memory.
//
// Shared memory layout: element i at sw(i) (spx_device.cuh), sw_len(M)
// elements per local FFT.  Twiddles are FP32 values of FP64-generated
// exponentials: tw_local holds, per pass p with radix R and stride Ns,
// W_{Ns R}^{r k} at [(r-1)*Ns + k] for r <= tw_rows(R) (radix 4: r = 1 only,
// and for Ns >= kTwSplitNs two factor tables, tw_split in spx_geom.h);
// tw_cross holds W_N^{n2} at [n2] (the cross stage forms W_N^{n2 k1} from it).
#pragma once

#include <cooperative_groups.h>
#include <cuda/atomic>

#include "spx.h"
#include "spx_device.cuh"
#include "spx_geom.h"

namespace spx {

namespace cg = cooperative_groups;

// Butterflies per thread needed by radix R when a thread owns <= EPT points.
template <int EPT, int R>
struct PassQ {
  static constexpr int value = (EPT + R - 1) / R;
};

// j mod Ns for the runtime stride of a pass, with magic = ceil(2^32 / Ns)
// (0 when Ns = 1): exact while j * Ns < 2^32 (j, Ns <= 16384 here).
SPX_DEV uint32_t mod_ns(uint32_t j, uint32_t Ns, uint32_t magic) {
  return magic ? j - Ns * __umulhi(j, magic) : 0u;
}

// Read-only load of a sample that is used once: not allocated in L1, so the
// stream of samples does not evict the twiddle tables the passes reuse.
SPX_DEV float2 ld_stream(const float2* p) {
  float2 v;
  asm volatile("ld.global.nc.L1::no_allocate.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "l"(p));
  return v;
}

// ---- window ------------------------------------------------------------------
// w[n], n < n_point, with the reference's (n_point - 1) denominator
// (pad_data_windowed, include/spectrum/kernels/fft_processor_kernels_rocm.hpp:97-110),
// c_k = cos(2 pi k n / (n_point - 1)):
//   Hann 0.5 - 0.5 c1 (evaluated as sin^2(pi n / (n_point - 1)), the same
//   value without the cancellation near the edges), Hamming 0.54 - 0.46 c1,
//   Blackman 0.42 - 0.5 c1 + 0.08 c2,
//   Blackman-Harris 0.35875 - 0.48829 c1 + 0.14128 c2 - 0.01168 c3.
// This one FP32 evaluation is the window of every path: the window table of
// the per-size kernels is filled by it on the device and the uneven batch
// calls it per sample, so both apply the same bits and give the same spectra.
// The argument is reduced exactly in integers: for an angle 2 pi m / D,
// 4 m = q D + r gives the quadrant q and the angle (pi/2) r / D, which folds
// to psi = (pi/2) s / D, s = min(r, D - r), psi in [0, pi/4]; (pi/2) / D is
// carried as a sum of two floats, so psi is within an ulp.  cos and sin of
// psi are their Taylor series (terms to psi^10 and psi^9; the first omitted
// terms are below 1.2e-10 and 2.5e-9 on [0, pi/4]) in Horner form with explicit
// FMAs, so no compiler contraction can change the bits.  Measured against
// FP64: Hann within 3 ulps of w everywhere, every window within 1.2e-7
// absolute (rounding the FP64 value to FP32 is within 3e-8).
struct WindowGen {
  uint32_t kind;   // spx_window (NONE when n_point < 2: w = 1)
  uint32_t D;      // n_point - 1
  float hi, lo;    // (pi/2) / D = hi + lo
};

SPX_DEV WindowGen make_window_gen(uint32_t kind, uint32_t n_point) {
  constexpr float kPio2Hi = 1.57079637050628662f;     // pi/2 rounded to FP32
  constexpr float kPio2Lo = -4.371139006309477e-8f;   // pi/2 - kPio2Hi
  WindowGen g;
  g.kind = n_point < 2 ? (uint32_t)SPX_WINDOW_NONE : kind;
  g.D = n_point < 2 ? 1u : n_point - 1u;
  const float d = __uint2float_rn(g.D);
  g.hi = __fdiv_rn(kPio2Hi, d);
  const float rem = __fmaf_rn(-g.hi, d, kPio2Hi);  // kPio2Hi - hi d, exact
  g.lo = __fdiv_rn(__fadd_rn(rem, kPio2Lo), d);
  return g;
}

// cos and sin of 2 pi m / D for m in [0, D), D < 2^29; (hi, lo) = (pi/2) / D.
SPX_DEV float2 sincos_turn(uint32_t m, uint32_t D, float hi, float lo) {
  const uint32_t m4 = 4u * m;
  const uint32_t q = (uint32_t)(m4 >= D) + (uint32_t)(m4 >= 2u * D) + (uint32_t)(m4 >= 3u * D);
  const uint32_t r = m4 - q * D;
  const bool swap = 2u * r > D;
  const float s = __uint2float_rn(swap ? D - r : r);
  const float psi = __fmaf_rn(s, hi, __fmul_rn(s, lo));
  const float y = __fmul_rn(psi, psi);
  // cos psi = 1 - y/2 + y^2/24 - y^3/720 + y^4/40320 - y^5/3628800
  float c = __fmaf_rn(y, -1.0f / 3628800.0f, 1.0f / 40320.0f);
  c = __fmaf_rn(c, y, -1.0f / 720.0f);
  c = __fmaf_rn(c, y, 1.0f / 24.0f);
  c = __fmaf_rn(c, y, -0.5f);
  c = __fmaf_rn(c, y, 1.0f);
  // sin psi = psi + psi y (-1/6 + y/120 - y^2/5040 + y^3/362880)
  float p = __fmaf_rn(y, 1.0f / 362880.0f, -1.0f / 5040.0f);
  p = __fmaf_rn(p, y, 1.0f / 120.0f);
  p = __fmaf_rn(p, y, -1.0f / 6.0f);
  const float sn = __fmaf_rn(__fmul_rn(psi, y), p, psi);
  // angle = q pi/2 + phi, phi = psi (or pi/2 - psi when folded)
  const float cphi = swap ? sn : c, sphi = swap ? c : sn;
  const float cv = (q & 1u) ? sphi : cphi, sv = (q & 1u) ? cphi : sphi;
  return make_float2((q == 1u || q == 2u) ? -cv : cv, (q >= 2u) ? -sv : sv);
}

// (k n) mod D for n <= D, k <= 3.
SPX_DEV uint32_t mul_mod(uint32_t k, uint32_t n, uint32_t D) {
  uint32_t m = k * n;
  m = m >= D ? m - D : m;
  m = m >= D ? m - D : m;
  m = m >= D ? m - D : m;
  return m;
}

SPX_DEV float cos_k(const WindowGen& g, uint32_t k, uint32_t n) {
  return sincos_turn(mul_mod(k, n, g.D), g.D, g.hi, g.lo).x;
}

SPX_DEV float window_at(const WindowGen& g, uint32_t n) {
  switch (g.kind) {
    case SPX_WINDOW_HANN: {  // sin(2 pi n / (2D)); (pi/2) / (2D) = (hi + lo) / 2 exactly
      const float s = sincos_turn(n, 2u * g.D, __fmul_rn(g.hi, 0.5f), __fmul_rn(g.lo, 0.5f)).y;
      return __fmul_rn(s, s);
    }
    case SPX_WINDOW_HAMMING: return __fmaf_rn(-0.46f, cos_k(g, 1, n), 0.54f);
    case SPX_WINDOW_BLACKMAN:
      return __fmaf_rn(0.08f, cos_k(g, 2, n), __fmaf_rn(-0.5f, cos_k(g, 1, n), 0.42f));
    case SPX_WINDOW_BLACKMAN_HARRIS:
      return __fmaf_rn(-0.01168f, cos_k(g, 3, n),
                       __fmaf_rn(0.14128f, cos_k(g, 2, n), __fmaf_rn(-0.48829f, cos_k(g, 1, n), 0.35875f)));
    default: return 1.0f;
  }
}

// Sample n of a beam: window applied (one rounded multiply per component,
// never fused into the butterfly that follows: every path gets the same
// windowed bits), zero beyond n_point.
SPX_DEV float2 load_sample(const float2* __restrict__ x, uint32_t n,
                           uint32_t n_point, const float* __restrict__ win) {
  float2 a = make_float2(0.f, 0.f);
  if (n < n_point) {
    a = ld_stream(x + n);
    if (win) {
      const float w = __ldg(win + n);
      a.x = __fmul_rn(a.x, w);
      a.y = __fmul_rn(a.y, w);
    }
  }
  return a;
}

// W_{4 Ns}^k of a radix-4 pass from its table t (tw_split layouts: two
// factors for Ns >= kTwSplitNs).
SPX_DEV float2 tw4(const float2* __restrict__ t, uint32_t k, uint32_t Ns) {
  return Ns >= kTwSplitNs ? cmul(__ldg(t + 64 + (k >> 6)), __ldg(t + (k & 63u))) : __ldg(t + k);
}

// One in-place Stockham pass over shared memory.  Loads all of a thread's
// butterflies, synchronises, computes, stores, synchronises.
template <int R, int Q>
SPX_DEV void pass_smem(float2* s, uint32_t M, uint32_t Ns, uint32_t magic,
                       const float2* __restrict__ tw, uint32_t tid, uint32_t T) {
  const uint32_t B = M / R;
  float2 v[Q][R];
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    const uint32_t j = tid + q * T;
    if (j < B) {
#pragma unroll
      for (int r = 0; r < R; ++r) v[q][r] = s[sw(j + r * B)];
    }
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    const uint32_t j = tid + q * T;
    if (j < B) {
      const uint32_t k = mod_ns(j, Ns, magic);
      if (Ns > 1) {
        if constexpr (R == 4) {
          const float2 w1 = tw4(tw, k, Ns), w2 = cmul(w1, w1);
          v[q][1] = cmul(v[q][1], w1); v[q][2] = cmul(v[q][2], w2); v[q][3] = cmul(v[q][3], cmul(w2, w1));
        } else {
#pragma unroll
          for (int r = 1; r < R; ++r) v[q][r] = cmul(v[q][r], __ldg(tw + (r - 1) * Ns + k));
        }
      }
      Dft<R>::run(v[q]);
      const uint32_t base = (j - k) * R + k;
#pragma unroll
      for (int r = 0; r < R; ++r) s[sw(base + r * Ns)] = v[q][r];
    }
  }
  __syncthreads();
}

// Loads sample n of a beam (window, zero padding) through the read-only path.
struct SampleLoader {
  const float2* __restrict__ x;
  uint32_t n_point;
  const float* __restrict__ win;
  SPX_DEV float2 operator()(uint32_t n) const { return load_sample(x, n, n_point, win); }
};

// Loads element n of a row written earlier in the same launch by other CTAs
// (the cluster exchange slot): L2-coherent loads, never the read-only path.
struct ExchangeLoader {
  const float2* row;
  SPX_DEV float2 operator()(uint32_t n) const { return __ldcg(row + n); }
};

// Output of a last local pass into a row of device memory: row[i] = Z[i]
// (L2-kept stores for rows read again in the same launch or the next one,
// streaming stores otherwise).
struct RowOut {
  float2* row;
  SPX_DEV void operator()(uint32_t i, float2 z) const { __stcg(row + i, z); }
};
struct RowOutStream {
  float2* row;
  SPX_DEV void operator()(uint32_t i, float2 z) const { __stcs(row + i, z); }
};

// First Stockham pass (Ns = 1) reading its inputs from device memory.
template <int R, int Q, typename Load>
SPX_DEV void pass_first_global(float2* s, uint32_t M, const Load& load, uint32_t tid, uint32_t T) {
  const uint32_t B = M / R;
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    const uint32_t j = tid + q * T;
    if (j < B) {
      float2 v[R];
#pragma unroll
      for (int r = 0; r < R; ++r) v[r] = load(j + r * B);
      Dft<R>::run(v);
#pragma unroll
      for (int r = 0; r < R; ++r) s[sw(j * R + r)] = v[r];
    }
  }
  __syncthreads();
}

template <int EPT, typename Load>
SPX_DEV void first_pass_dispatch(float2* s, const FftGeom& g, const Load& load, uint32_t tid,
                                 uint32_t T) {
  switch (g.radix[0]) {
    case 16: pass_first_global<16, PassQ<EPT, 16>::value>(s, g.M, load, tid, T); break;
    case 9: pass_first_global<9, PassQ<EPT, 9>::value>(s, g.M, load, tid, T); break;
    case 8: pass_first_global<8, PassQ<EPT, 8>::value>(s, g.M, load, tid, T); break;
    case 6: pass_first_global<6, PassQ<EPT, 6>::value>(s, g.M, load, tid, T); break;
    case 4: pass_first_global<4, PassQ<EPT, 4>::value>(s, g.M, load, tid, T); break;
    case 3: pass_first_global<3, PassQ<EPT, 3>::value>(s, g.M, load, tid, T); break;
    default: pass_first_global<2, PassQ<EPT, 2>::value>(s, g.M, load, tid, T); break;
  }
}

// Cross-CTA stage through device memory: CTA `c` computes the CR-point DFTs
// of its slice of n2, applies W_N^{n2 k1} and writes element k1 to
// slot[k1*M + n2] (L2-resident exchange slot of its cluster).  The caller
// separates this from the reads of the slot with a cluster barrier.
// W_N^{n2 k1} is W_N^{n2} (one table load: tw_cross holds W_N^{n2}, n2 < M)
// raised by a product tree (w^k = (w^{k/2})^2 for even k, w^{k-1} w for odd
// k; at most 2 log2 C deep): six loads per column fewer for C = 8 (the
// headline step 0.2825 -> 0.2782 ms), a few ulps of twiddle error.  A chain
// of successive products measured the same on the headline and 2 % slower
// on the uneven batch (cross stages of 6 and 9).
template <int CR>
SPX_DEV void cross_stage_exchange(float2* __restrict__ slot, uint32_t c, uint32_t M,
                                  const SampleLoader& load, const float2* __restrict__ twc,
                                  uint32_t tid, uint32_t T) {
  const uint32_t S = (M + CR - 1) / CR;
  const uint32_t lo = c * S;
  const uint32_t hi = min(lo + S, M);
#pragma unroll 2
  for (uint32_t n2 = lo + tid; n2 < hi; n2 += T) {
    float2 v[CR];
#pragma unroll
    for (int n1 = 0; n1 < CR; ++n1) v[n1] = load(n1 * M + n2);
    Dft<CR>::run(v);
    __stcg(slot + n2, v[0]);
    float2 w[CR];
    w[1] = __ldg(twc + n2);
#pragma unroll
    for (int k1 = 2; k1 < CR; ++k1) w[k1] = (k1 % 2 == 0) ? cmul(w[k1 / 2], w[k1 / 2]) : cmul(w[k1 - 1], w[1]);
#pragma unroll
    for (int k1 = 1; k1 < CR; ++k1) __stcg(slot + (size_t)k1 * M + n2, cmul(v[k1], w[k1]));
  }
}

// Starts asynchronous L2 fills of the 16-byte granules lying entirely in
// [p, p + bytes), in 16 KB pieces spread over threads tid, tid + T, ...
// (cp.async.bulk.prefetch: no result, no ordering; the range must be valid
// device memory).
SPX_DEV void prefetch_l2(const void* p, size_t bytes, uint32_t tid, uint32_t T) {
  constexpr uintptr_t kPiece = 16384;
  const uintptr_t a = reinterpret_cast<uintptr_t>(p);
  const uintptr_t lo = (a + 15) & ~(uintptr_t)15;
  const uintptr_t hi = (a + bytes) & ~(uintptr_t)15;
  for (uintptr_t x = lo + (uintptr_t)tid * kPiece; x < hi; x += (uintptr_t)T * kPiece) {
    const uint32_t n = (uint32_t)min(kPiece, hi - x);
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(x), "r"(n) : "memory");
  }
}

// Prefetch into L2 of the samples of beam `beam + g.ahead` that this CTA
// will read when it runs that beam's turn one residency wave later: the whole
// beam (C == 1) or, for rank c of a cluster, the C slices [n1 M + c S,
// n1 M + c S + S) of its cross stage.
// The samples of an n_point-sample beam x that rank c of its C CTAs reads
// first (the whole beam for C == 1, the cross-stage slices otherwise).
SPX_DEV void prefetch_beam_part(const float2* x, uint32_t n_point, uint32_t C, uint32_t M, uint32_t c,
                                uint32_t tid, uint32_t T) {
  if (C == 1) {
    prefetch_l2(x, (size_t)n_point * sizeof(float2), tid, T);
    return;
  }
  const uint32_t S = (M + C - 1) / C;
  if (tid < C) {
    const uint32_t lo = tid * M + c * S;
    const uint32_t hi = min(min(lo + S, (tid + 1) * M), n_point);
    if (lo < hi) prefetch_l2(x + lo, (size_t)(hi - lo) * sizeof(float2), 0, 1);
  }
}

SPX_DEV void prefetch_future_beam(const FftGeom& g, const float2* in, uint32_t n_point, uint32_t beam,
                                  uint32_t c, uint32_t tid, uint32_t T) {
  if (g.ahead == 0 || beam + g.ahead >= g.beams) return;
  prefetch_beam_part(in + (size_t)(beam + g.ahead) * n_point, n_point, g.C, g.M, c, tid, T);
}

// Invalidates (without write-back) every 128-byte L2 line lying entirely in
// [p, p + bytes); lines shared with a neighbouring row are left alone.
SPX_DEV void discard_row_l2(const float2* p, size_t bytes, uint32_t tid, uint32_t T) {
  const uintptr_t a = reinterpret_cast<uintptr_t>(p);
  const uintptr_t lo = (a + 127) & ~(uintptr_t)127;
  const uintptr_t hi = (a + bytes) & ~(uintptr_t)127;
  for (uintptr_t x = lo + (uintptr_t)tid * 128; x < hi; x += (uintptr_t)T * 128)
    asm volatile("discard.global.L2 [%0], 128;" ::"l"(x) : "memory");
}

// Barrier of the C CTAs working on one beam (one cooperative launch, so all
// CTAs are resident), in two halves so that a CTA can work between them:
// group_arrive adds this CTA's arrival to the beam's counter; group_wait
// waits until C have arrived (acquire), at most kSpinLimitNs, then sets
// kErrLookbackTimeout and goes on.  As in a grid-wide barrier, the CTA
// barrier orders every thread's prior writes before thread 0's device-scope
// fence and release, so only thread 0 fences.
SPX_DEV void group_arrive(uint32_t* count) {
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    cuda::atomic_ref<uint32_t, cuda::thread_scope_device> r(*count);
    r.fetch_add(1u, cuda::memory_order_release);
  }
}

SPX_DEV void group_wait(uint32_t* count, uint32_t C, uint32_t* err) {
  if (threadIdx.x == 0) {
    cuda::atomic_ref<uint32_t, cuda::thread_scope_device> r(*count);
    if (r.load(cuda::memory_order_acquire) < C) {
      const uint64_t t0 = globaltimer_ns();
      while (r.load(cuda::memory_order_acquire) < C) {
        if (globaltimer_ns() - t0 > kSpinLimitNs) {
          atomicOr(err, kErrLookbackTimeout);
          break;
        }
      }
    }
  }
  __syncthreads();
}

SPX_DEV void group_barrier(uint32_t* count, uint32_t C, uint32_t* err) {
  group_arrive(count);
  group_wait(count, C, err);
}

// Runs the passes p, p+1, ... while they have radix R; returns the next pass.
template <int R, int EPT>
SPX_DEV uint32_t run_radix(float2* s, const FftGeom& g, uint32_t p,
                           const float2* __restrict__ tw_local, uint32_t tid, uint32_t T) {
  while (p < g.npass && g.radix[p] == R) {
    pass_smem<R, PassQ<EPT, R>::value>(s, g.M, g.ns[p], g.nsmagic[p], tw_local + g.twoff[p], tid, T);
    ++p;
  }
  return p;
}

// Runs local passes p0.. of the plan.  Passes run as consecutive runs of
// equal radix in the fixed order the plan builder emits (8, 16..., 9..., 3,
// 4, 2); one loop per radix keeps the register allocation of each pass
// separate (a switch inside a single pass loop spills).
template <int EPT>
SPX_DEV void local_passes(float2* s, const FftGeom& g, uint32_t p0,
                          const float2* __restrict__ tw_local, uint32_t tid, uint32_t T) {
  uint32_t p = p0;
  p = run_radix<8, EPT>(s, g, p, tw_local, tid, T);
  p = run_radix<16, EPT>(s, g, p, tw_local, tid, T);
  p = run_radix<9, EPT>(s, g, p, tw_local, tid, T);
  p = run_radix<3, EPT>(s, g, p, tw_local, tid, T);
  p = run_radix<4, EPT>(s, g, p, tw_local, tid, T);
  p = run_radix<2, EPT>(s, g, p, tw_local, tid, T);
}

// ---------------------------------------------------------------------------
// Compile-time plans for local sizes M = 2^a 3^b <= 16384 (EPT = 16).  The
// radix order, strides and twiddle offsets are those build_geom emits (an 8
// first when a = 3 mod 4, then 16s, 9s, a 3 when b is odd, a 4 or 2 last),
// so the plan's twiddle table is used unchanged and the results are
// bit-identical to the runtime passes; only the index arithmetic becomes
// constant.  The CTA has T threads (by default ceil(M / 16) rounded up to a
// warp, the runtime plan's count): a pass of radix R has B = M / R
// butterflies, Q = ceil(B / T) per thread, the last one guarded when T does
// not divide B.  Which thread computes a butterfly does not change its
// arithmetic, so any T gives the same bits.
// ---------------------------------------------------------------------------
constexpr int ct_v2(int m) { return m % 2 ? 0 : 1 + ct_v2(m / 2); }
constexpr int ct_v3(int m) { return m % 3 ? 0 : 1 + ct_v3(m / 3); }
constexpr int ct_pow3(int e) { return e == 0 ? 1 : 3 * ct_pow3(e - 1); }

template <int M>
struct CtPlan {
  static constexpr int a = ct_v2(M), b = ct_v3(M);
  static constexpr bool lead8 = a % 4 == 3;
  static constexpr int n16 = a / 4, n9 = b / 2, n3 = b % 2;
  static constexpr int tail = lead8 ? 1 : (1 << (a % 4));  // last radix 2 or 4, 1 = none
  static constexpr int npass = (lead8 ? 1 : 0) + n16 + n9 + n3 + (tail > 1 ? 1 : 0);
  static constexpr int T = (((M + 15) / 16) + 31) / 32 * 32;
  static constexpr int radix(int p) {
    return lead8 && p == 0 ? 8
         : (p - (lead8 ? 1 : 0)) < n16 ? 16
         : (p - (lead8 ? 1 : 0) - n16) < n9 ? 9
         : (p - (lead8 ? 1 : 0) - n16 - n9) < n3 ? 3
         : tail;
  }
  static constexpr int ns(int p) { return p == 0 ? 1 : ns(p - 1) * radix(p - 1); }
  static constexpr int twoff(int p) {
    return p == 0 ? 0 : twoff(p - 1) + (int)tw_entries((uint32_t)radix(p - 1), (uint32_t)ns(p - 1));
  }
  static_assert(M == (1 << a) * ct_pow3(b) && M <= 16384, "M must be 2^a 3^b <= 16384");
};

// First pass (Ns = 1) from `load`, results into shared memory.
template <int M, int T = CtPlan<M>::T, typename Load>
SPX_DEV void ct_first(float2* s, const Load& load, uint32_t tid) {
  using P = CtPlan<M>;
  constexpr int R = P::radix(0), B = M / R, Q = (B + T - 1) / T;
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    const uint32_t j = tid + q * T;
    if (B % T == 0 || q + 1 < Q || j < (uint32_t)B) {
      float2 v[R];
#pragma unroll
      for (int r = 0; r < R; ++r) v[r] = load(j + r * B);
      Dft<R>::run(v);
      if constexpr (16 % R == 0) {
        // base = R j: base mod 16 + r < 16, so sw(base + r) = sw(base) + r
        const uint32_t sb = sw(j * R);
#pragma unroll
        for (int r = 0; r < R; ++r) s[sb + r] = v[r];
      } else {
#pragma unroll
        for (int r = 0; r < R; ++r) s[sw(j * R + r)] = v[r];
      }
    }
  }
  __syncthreads();
}

// Pass P >= 1 in shared memory.  The last pass (Ns = M / R = B) writes each
// butterfly's outputs to the elements it read (base = j), so it needs no
// barrier between its loads and its stores.
template <int M, int P, int T>
SPX_DEV void ct_pass(float2* s, const float2* __restrict__ tw, uint32_t tid) {
  using PL = CtPlan<M>;
  constexpr int R = PL::radix(P), Ns = PL::ns(P), B = M / R, Q = (B + T - 1) / T;
  float2 v[Q][R];
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    const uint32_t j = tid + q * T;
    if (B % T == 0 || q + 1 < Q || j < (uint32_t)B) {
      const uint32_t sj = sw(j);
#pragma unroll
      for (int r = 0; r < R; ++r) v[q][r] = s[(B % 16 == 0) ? sj + sw(r * B) : sw(j + r * B)];
    }
  }
  if constexpr (P + 1 < PL::npass) __syncthreads();
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    const uint32_t j = tid + q * T;
    if (B % T == 0 || q + 1 < Q || j < (uint32_t)B) {
      const uint32_t k = j % Ns;
      const float2* t = tw + PL::twoff(P) + k;
      if constexpr (R == 4) {
        const float2 w1 = tw4(tw + PL::twoff(P), k, Ns), w2 = cmul(w1, w1);
        v[q][1] = cmul(v[q][1], w1); v[q][2] = cmul(v[q][2], w2); v[q][3] = cmul(v[q][3], cmul(w2, w1));
      } else {
#pragma unroll
        for (int r = 1; r < R; ++r) v[q][r] = cmul(v[q][r], __ldg(t + (r - 1) * Ns));
      }
      Dft<R>::run(v[q]);
      const uint32_t base = (j - k) * R + k;
      const uint32_t sb = sw(base);
#pragma unroll
      for (int r = 0; r < R; ++r) s[(Ns % 16 == 0) ? sb + sw(r * Ns) : sw(base + r * Ns)] = v[q][r];
    }
  }
  __syncthreads();
}

template <int M, int P, int T>
SPX_DEV void ct_passes_from(float2* s, const float2* __restrict__ tw, uint32_t tid) {
  if constexpr (P < CtPlan<M>::npass) {
    ct_pass<M, P, T>(s, tw, tid);
    ct_passes_from<M, P + 1, T>(s, tw, tid);
  }
}

// The last pass (P = npass - 1 >= 1) with its outputs handed to out(i, z)
// (element i of the local FFT's natural-order result) instead of shared
// memory: consecutive threads get consecutive i, so a store to a row in
// device memory is coalesced.  Ends without a barrier.
template <int M, int T, typename Out>
SPX_DEV void ct_last_pass_out(const float2* s, const float2* __restrict__ tw, uint32_t tid, const Out& out) {
  using PL = CtPlan<M>;
  constexpr int P = PL::npass - 1;
  constexpr int R = PL::radix(P), Ns = PL::ns(P), B = M / R, Q = (B + T - 1) / T;
  static_assert(P >= 1 && Ns == B, "the last pass of the plan");
  float2 v[Q][R];
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    const uint32_t j = tid + q * T;
    if (B % T == 0 || q + 1 < Q || j < (uint32_t)B) {
      const uint32_t sj = sw(j);
#pragma unroll
      for (int r = 0; r < R; ++r) v[q][r] = s[(B % 16 == 0) ? sj + sw(r * B) : sw(j + r * B)];
    }
  }
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    const uint32_t j = tid + q * T;
    if (B % T == 0 || q + 1 < Q || j < (uint32_t)B) {
      const float2* t = tw + PL::twoff(P) + j;  // k = j mod Ns = j
      if constexpr (R == 4) {
        const float2 w1 = tw4(tw + PL::twoff(P), j, Ns), w2 = cmul(w1, w1);
        v[q][1] = cmul(v[q][1], w1); v[q][2] = cmul(v[q][2], w2); v[q][3] = cmul(v[q][3], cmul(w2, w1));
      } else {
#pragma unroll
        for (int r = 1; r < R; ++r) v[q][r] = cmul(v[q][r], __ldg(t + (r - 1) * Ns));
      }
      Dft<R>::run(v[q]);
#pragma unroll
      for (int r = 0; r < R; ++r) out(j + r * B, v[q][r]);
    }
  }
}

template <int M, int P, int T>
SPX_DEV void ct_passes_until_last(float2* s, const float2* __restrict__ tw, uint32_t tid) {
  if constexpr (P + 1 < CtPlan<M>::npass) {
    ct_pass<M, P, T>(s, tw, tid);
    ct_passes_until_last<M, P + 1, T>(s, tw, tid);
  }
}

// Whole local FFT of M points (first pass from `load`) by a CTA of T
// threads, ending with a barrier.
template <int M, int T = CtPlan<M>::T, typename Load>
SPX_DEV void ct_local_fft(float2* s, const Load& load, const float2* __restrict__ tw, uint32_t tid) {
  ct_first<M, T>(s, load, tid);
  ct_passes_from<M, 1, T>(s, tw, tid);
}

// The local FFT of ct_local_fft with the last pass's outputs handed to
// out(i, z) (ct_last_pass_out) instead of shared memory; ends without a
// barrier (the shared memory is still being read by the last pass).
template <int M, int T = CtPlan<M>::T, typename Load, typename Out>
SPX_DEV void ct_local_fft_out(float2* s, const Load& load, const float2* __restrict__ tw, uint32_t tid,
                              const Out& out) {
  static_assert(CtPlan<M>::npass >= 2, "at least one pass after the first");
  ct_first<M, T>(s, load, tid);
  ct_passes_until_last<M, 1, T>(s, tw, tid);
  ct_last_pass_out<M, T>(s, tw, tid, out);
}

// The local sizes with an out-of-line compile-time plan (kernels that take
// many sizes call them through ct_menu_fft; one register allocation each).
// Together they cover every 2^a 3^b transform of 16385 .. 262144 points as
// C x M with C in {2, 3, 4, 6, 8, 9, 12, 16}, each at the largest such M.
template <int M, int T, typename Load, typename Out>
__device__ __noinline__ void ct_local_fft_ool(float2* s, Load load, const float2* __restrict__ tw, uint32_t tid,
                                              Out out) {
  ct_local_fft_out<M, T>(s, load, tw, tid, out);
}

// The compile-time local FFT of M points, its last pass's outputs handed to
// out(i, z), when M is in the menu (returns true), else nothing (returns
// false).  The CTA has T threads, or the plan's default count when T = 0.
template <int T, typename Load, typename Out>
SPX_DEV bool ct_menu_fft(uint32_t M, float2* s, const Load& load, const float2* __restrict__ tw, uint32_t tid,
                         const Out& out) {
  switch (M) {
    case 4096: ct_local_fft_ool<4096, T ? T : CtPlan<4096>::T>(s, load, tw, tid, out); return true;
    case 5832: ct_local_fft_ool<5832, T ? T : CtPlan<5832>::T>(s, load, tw, tid, out); return true;
    case 6144: ct_local_fft_ool<6144, T ? T : CtPlan<6144>::T>(s, load, tw, tid, out); return true;
    case 6561: ct_local_fft_ool<6561, T ? T : CtPlan<6561>::T>(s, load, tw, tid, out); return true;
    case 8192: ct_local_fft_ool<8192, T ? T : CtPlan<8192>::T>(s, load, tw, tid, out); return true;
    case 8748: ct_local_fft_ool<8748, T ? T : CtPlan<8748>::T>(s, load, tw, tid, out); return true;
    case 9216: ct_local_fft_ool<9216, T ? T : CtPlan<9216>::T>(s, load, tw, tid, out); return true;
    case 10368: ct_local_fft_ool<10368, T ? T : CtPlan<10368>::T>(s, load, tw, tid, out); return true;
    case 11664: ct_local_fft_ool<11664, T ? T : CtPlan<11664>::T>(s, load, tw, tid, out); return true;
    case 12288: ct_local_fft_ool<12288, T ? T : CtPlan<12288>::T>(s, load, tw, tid, out); return true;
    case 13122: ct_local_fft_ool<13122, T ? T : CtPlan<13122>::T>(s, load, tw, tid, out); return true;
    case 13824: ct_local_fft_ool<13824, T ? T : CtPlan<13824>::T>(s, load, tw, tid, out); return true;
    case 15552: ct_local_fft_ool<15552, T ? T : CtPlan<15552>::T>(s, load, tw, tid, out); return true;
    case 16384: ct_local_fft_ool<16384, T ? T : CtPlan<16384>::T>(s, load, tw, tid, out); return true;
    default: return false;
  }
}

// Runs the local FFT with the compile-time plan when g is a power-of-two
// size it covers inline (EPT 16, one thread per 16 points), else the runtime
// plan.  Returns after the last pass's barrier either way.
template <int EPT, typename Load>
SPX_DEV void local_fft(float2* s, const FftGeom& g, const Load& load, const float2* __restrict__ tw,
                       uint32_t tid, uint32_t T) {
  if constexpr (EPT == 16) {
    if (g.M == 16384 && T == 1024) return ct_local_fft<16384>(s, load, tw, tid);
    if (g.M == 8192 && T == 512) return ct_local_fft<8192>(s, load, tw, tid);
    if (g.M == 4096 && T == 256) return ct_local_fft<4096>(s, load, tw, tid);
  }
  first_pass_dispatch<EPT>(s, g, load, tid, T);
  local_passes<EPT>(s, g, 1, tw, tid, T);
}

// local_fft with the natural-order result handed to out(i, z), i < M: from
// the last pass's registers for the compile-time plans, else read back from
// shared memory after the last pass.  Ends without a barrier.
template <int EPT, typename Load, typename Out>
SPX_DEV void local_fft_out(float2* s, const FftGeom& g, const Load& load, const float2* __restrict__ tw,
                           uint32_t tid, uint32_t T, const Out& out) {
  if constexpr (EPT == 16) {
    if (g.M == 16384 && T == 1024) return ct_local_fft_out<16384>(s, load, tw, tid, out);
    if (g.M == 8192 && T == 512) return ct_local_fft_out<8192>(s, load, tw, tid, out);
    if (g.M == 4096 && T == 256) return ct_local_fft_out<4096>(s, load, tw, tid, out);
  }
  first_pass_dispatch<EPT>(s, g, load, tid, T);
  local_passes<EPT>(s, g, 1, tw, tid, T);
  for (uint32_t i = tid; i < g.M; i += T) out(i, s[sw(i)]);
}

// Output modes of the inverse and real-input transforms (beyond spx_fft_out).
constexpr uint32_t kOutComplexReversed = 16;  // out[(nfft - k) mod nfft] = X[k] * scale
constexpr uint32_t kOutR2CHalf = 17;          // k <= nfft/2: out[beam (nfft/2 + 1) + k] = X[k]
constexpr uint32_t kOutR2CFull = 18;          // k <= nfft/2: X[k] at k, conj(X[k]) at nfft - k

// Writes bin k (= X[k]) of one beam in output mode `out_mode` (the layouts of
// epilogue_out below).
SPX_DEV void store_bin(void* __restrict__ out, uint32_t out_mode, float scale, const FftGeom& g,
                       uint32_t beam, uint32_t k, float2 z) {
  const size_t obase = (size_t)beam * g.nfft;
  const uint32_t half = g.nfft / 2;
  switch (out_mode) {
    case SPX_OUT_COMPLEX: reinterpret_cast<float2*>(out)[obase + k] = z; break;
    case SPX_OUT_MAG: reinterpret_cast<float*>(out)[obase + k] = __fmul_rn(mag_rn(z), scale); break;
    case SPX_OUT_MAG2: reinterpret_cast<float*>(out)[obase + k] = __fmul_rn(mag2_rn(z), scale); break;
    case SPX_OUT_MAGPHASE:
      reinterpret_cast<float2*>(out)[obase + k] = make_float2(mag_rn(z), atan2f(z.y, z.x));
      break;
    case kOutComplexReversed:
      reinterpret_cast<float2*>(out)[obase + (k == 0 ? 0u : g.nfft - k)] =
          make_float2(__fmul_rn(z.x, scale), __fmul_rn(z.y, scale));
      break;
    case kOutR2CHalf:
      if (k <= half) reinterpret_cast<float2*>(out)[(size_t)beam * (half + 1) + k] = z;
      break;
    default:  // kOutR2CFull
      if (k <= half) {
        float2* o = reinterpret_cast<float2*>(out) + obase;
        o[k] = z;
        if (k >= 1 && k < g.nfft - half) o[g.nfft - k] = make_float2(z.x, -z.y);
      }
      break;
  }
}

// Output of bin k = i of one beam's natural-order spectrum (C = 1) in any
// output mode (the layouts of store_bin), for local_fft_out.
struct BinOut {
  void* out;
  uint32_t out_mode;
  float scale;
  const FftGeom* g;
  uint32_t beam;
  SPX_DEV void operator()(uint32_t i, float2 z) const { store_bin(out, out_mode, scale, *g, beam, i, z); }
};

}  // namespace spx
