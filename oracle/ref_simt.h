// ref_simt.h — a minimal CPU executor for CUDA/HIP-style kernel source.
//
// TEST INFRASTRUCTURE ONLY (oracle pinning).  It lets the reference's own
// device-kernel text, extracted from its headers at build time into
// oracle/_ref/, run on the host so the numpy restatement can be checked
// against the reference's exact arithmetic and reduction order.
//
// Model: one block at a time; every thread of the block is a ucontext
// fiber.  __syncthreads() yields to the scheduler, which resumes the fibers
// round-robin, so a barrier completes once every live thread reached it
// (valid for kernels whose threads all pass the same barriers, as the
// reference's kernels do).  __shared__ variables become function-static,
// i.e. shared by the fibers of the block that is running.
#pragma once

#include <ucontext.h>

#include <cmath>
#include <cstddef>
#include <cstdint>
#include <functional>
#include <vector>

struct ref_uint3 {
  unsigned int x, y, z;
};

extern ref_uint3 threadIdx, blockIdx, blockDim, gridDim;
void __syncthreads();
void* ref_simt_dynamic_smem();

#define __global__
#define __device__
#define __host__
#define __forceinline__ inline
#define __shared__ static
#define __launch_bounds__(...)

inline float __fsqrt_rn(float x) { return std::sqrt(x); }
inline float __cosf(float x) { return std::cos(x); }

namespace ref_simt {

// Runs body() for every thread of every block of the grid.
void launch(ref_uint3 grid, ref_uint3 block, size_t dyn_smem_bytes,
            const std::function<void()>& body);

inline ref_uint3 dim(unsigned x, unsigned y = 1, unsigned z = 1) { return ref_uint3{x, y, z}; }

}  // namespace ref_simt
