// Vector kernels of the flexible GMRES outer iteration (sm_103a).
//
// Block Gram-Schmidt needs, per Arnoldi step j, the j+1 dot products of the
// new vector w with the basis V_0..V_j and the update w -= sum_i h_i V_i.
// k_mdot reads w once per basis vector from L2 and writes per-block partial
// sums; k_mdot_finish adds each dot's partials in block order (one block per
// dot, the same order every run, so results are bit-reproducible);
// k_maxpy applies the j+1 coefficients in index order.  The basis is one
// array of cnt vectors of n doubles at a stride of ld.
#include "gbmg_internal.h"

namespace gbmg {

namespace {

constexpr int kMThreads = 256;

template <int NV>
__device__ __forceinline__ double block_sum1(double v, double* ws) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if (lane == 0) ws[wid] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x == 0)
    for (int w = 0; w < NV; ++w) t += ws[w];
  __syncthreads();
  return t;
}

__global__ void __launch_bounds__(kMThreads) k_mdot(const double* __restrict__ V, size_t ld, int cnt,
                                                    const double* __restrict__ w, size_t n,
                                                    double* __restrict__ partials) {
  __shared__ double ws[kMThreads / 32];
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (int i = 0; i < cnt; ++i) {
    const double* vi = V + (size_t)i * ld;
    double acc = 0.0;
    for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += stride)
      acc += vi[q] * w[q];
    const double t = block_sum1<kMThreads / 32>(acc, ws);
    if (threadIdx.x == 0) partials[(size_t)i * gridDim.x + blockIdx.x] = t;
  }
}

__global__ void __launch_bounds__(kMThreads) k_mdot_finish(const double* __restrict__ partials,
                                                           int blocks, double* __restrict__ out) {
  __shared__ double ws[kMThreads / 32];
  const int i = blockIdx.x;
  double acc = 0.0;
  for (int b = threadIdx.x; b < blocks; b += blockDim.x) acc += partials[(size_t)i * blocks + b];
  const double t = block_sum1<kMThreads / 32>(acc, ws);
  if (threadIdx.x == 0) out[i] = t;
}

// w += sign * sum_i coef[i] V_i
__global__ void __launch_bounds__(kMThreads) k_maxpy(double* __restrict__ w,
                                                     const double* __restrict__ V, size_t ld,
                                                     const double* __restrict__ coef, int cnt,
                                                     double sign, size_t n) {
  for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < n;
       q += (size_t)gridDim.x * blockDim.x) {
    double acc = 0.0;
    for (int i = 0; i < cnt; ++i) acc += coef[i] * V[(size_t)i * ld + q];
    w[q] += sign * acc;
  }
}

// out may be in (scaling in place)
__global__ void __launch_bounds__(kMThreads) k_scale_copy(double* out, const double* in,
                                                          double alpha, size_t n) {
  for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < n;
       q += (size_t)gridDim.x * blockDim.x)
    out[q] = alpha * in[q];
}

// w *= 1/sqrt(*nrm2) (w unchanged when the norm is 0)
__global__ void __launch_bounds__(kMThreads) k_scale_rsqrt(double* w, const double* nrm2,
                                                           size_t n) {
  const double v = *nrm2;
  if (!(v > 0.0)) return;
  const double a = 1.0 / sqrt(v);
  for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < n;
       q += (size_t)gridDim.x * blockDim.x)
    w[q] = a * w[q];
}

unsigned grid_for(size_t n, int max_blocks) {
  size_t b = (n + kMThreads - 1) / kMThreads;
  if (b > (size_t)max_blocks) b = (size_t)max_blocks;
  return (unsigned)(b > 0 ? b : 1);
}

}  // namespace

void launch_mdot(cudaStream_t s, const double* V, size_t ld, int cnt, const double* w, size_t n,
                 double* partials, int max_blocks, double* out) {
  const unsigned g = grid_for(n, max_blocks);
  k_mdot<<<g, kMThreads, 0, s>>>(V, ld, cnt, w, n, partials);
  k_mdot_finish<<<(unsigned)cnt, kMThreads, 0, s>>>(partials, (int)g, out);
}

void launch_maxpy(cudaStream_t s, double* w, const double* V, size_t ld, const double* coef,
                  int cnt, double sign, size_t n) {
  k_maxpy<<<grid_for(n, 4096), kMThreads, 0, s>>>(w, V, ld, coef, cnt, sign, n);
}

void launch_scale_copy(cudaStream_t s, double* out, const double* in, double alpha, size_t n) {
  k_scale_copy<<<grid_for(n, 4096), kMThreads, 0, s>>>(out, in, alpha, n);
}

void launch_scale_rsqrt(cudaStream_t s, double* w, const double* nrm2, size_t n) {
  k_scale_rsqrt<<<grid_for(n, 4096), kMThreads, 0, s>>>(w, nrm2, n);
}

}  // namespace gbmg
