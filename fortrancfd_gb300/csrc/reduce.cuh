// Deterministic single-pass grid reductions in FP64.
//
// Each block reduces its values with warp shuffles and one shared-memory
// step, writes its partial sums to ReduceScratch::partials[block], and bumps
// the completion counter.  The block that arrives last sums all partials in a
// fixed order, stores the result slot and resets the counter to 0, so a
// reduction costs one launch and gives bit-identical results run to run.
#pragma once

#include "gbmg_internal.h"

namespace gbmg {

constexpr int kRedThreads = 256;

// Grid-stride traversal of [0, n) that loads four strided elements (q, q+s,
// q+2s, q+3s) before using any, so their memory requests are in flight
// together; use(q, v) runs in the same order as in a one-at-a-time loop, so
// sums come out bit for bit the same.
template <typename Load, typename Use>
__device__ __forceinline__ void stride4(size_t n, Load load, Use use) {
  const size_t s = (size_t)gridDim.x * blockDim.x;
  size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  for (; q + 3 * s < n; q += 4 * s) {
    const auto v0 = load(q);
    const auto v1 = load(q + s);
    const auto v2 = load(q + 2 * s);
    const auto v3 = load(q + 3 * s);
    use(q, v0);
    use(q + s, v1);
    use(q + 2 * s, v2);
    use(q + 3 * s, v3);
  }
  for (; q < n; q += s) use(q, load(q));
}

// Sum over the block of NV values; the result is valid in thread 0.
template <int NV>
__device__ inline void block_sum(double (&v)[NV]) {
  __shared__ double ws[NV][kRedThreads / 32];
  const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
  const int lane = tid & 31, wid = tid >> 5;
  const int nwarps = (blockDim.x * blockDim.y * blockDim.z + 31) >> 5;
#pragma unroll
  for (int c = 0; c < NV; ++c) {
    double x = v[c];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) ws[c][wid] = x;
  }
  __syncthreads();
  if (wid == 0) {
#pragma unroll
    for (int c = 0; c < NV; ++c) {
      double x = lane < nwarps ? ws[c][lane] : 0.0;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
      v[c] = x;
    }
  }
  __syncthreads();
}

// Finish a grid reduction of NV values into R.result[slot .. slot+NV-1].
// Every thread of every block must call this exactly once.
template <int NV>
__device__ inline void grid_sum_finish(double (&v)[NV], const ReduceScratch& R, int slot) {
  __shared__ bool am_last;
  const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
  const int nthreads = blockDim.x * blockDim.y * blockDim.z;
  const unsigned int bid = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
  const unsigned int nblocks = gridDim.x * gridDim.y * gridDim.z;
  block_sum<NV>(v);
  if (tid == 0) {
#pragma unroll
    for (int c = 0; c < NV; ++c) R.partials[(size_t)c * R.max_blocks + bid] = v[c];
    __threadfence();
    const unsigned int t = atomicAdd(R.counter, 1u);
    am_last = (t == nblocks - 1);
  }
  __syncthreads();
  if (am_last) {
    __threadfence();
    double w[NV];
#pragma unroll
    for (int c = 0; c < NV; ++c) {
      double acc = 0.0;
      for (unsigned int b = tid; b < nblocks; b += nthreads)
        acc += __ldcg(&R.partials[(size_t)c * R.max_blocks + b]);
      w[c] = acc;
    }
    block_sum<NV>(w);
    if (tid == 0) {
#pragma unroll
      for (int c = 0; c < NV; ++c) R.result[slot + c] = w[c];
      *R.counter = 0u;
    }
  }
}

}  // namespace gbmg
