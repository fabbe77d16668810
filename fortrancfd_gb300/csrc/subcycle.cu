// The bottom of the V-cycle in one thread block (sm_103a).
//
// Levels with at most kSubMaxCells cells are launch-latency bound: a sweep of
// 16^3 cells is a few microseconds of launch and drain for nanoseconds of
// work.  This kernel runs everything from level lc down and back up --
// sweeps, residual + restriction, the dense coarsest solve, prolongation --
// in one block, with every level's unknown, right-hand side and face
// coefficients in shared memory (the coefficients are staged once at the
// start, so no phase waits on L2).  Phases are separated by __syncthreads().  Each step does the arithmetic of the corresponding
// separate kernel in the same order (red-black update, children summed in z,
// y, x order, slopes added x, y, z), so the cycle is the same cycle.
#include "gbmg_internal.h"
#include "mg_cells.cuh"
#include "pdl.cuh"

namespace gbmg {

namespace {

constexpr int kSubThreads = 1024;

template <typename T>
__device__ __forceinline__ void sub_stencil(const SubLevel<T>& L, const T* __restrict__ p, int i,
                                            int j, int k, int q, T& s, T& d) {
  const int sy = L.nx, sz = L.nx * L.ny;
  T c;
  s = T(0);
  d = T(0);
  if (i > 0) { c = L.cx[q]; s += c * p[q - 1]; d += c; }
  if (i < L.nx - 1) { c = L.cx[q + 1]; s += c * p[q + 1]; d += c; }
  if (j > 0) { c = L.cy[q]; s += c * p[q - sy]; d += c; }
  if (j < L.ny - 1) { c = L.cy[q + sy]; s += c * p[q + sy]; d += c; }
  if (k > 0) { c = L.cz[q]; s += c * p[q - sz]; d += c; }
  if (k < L.nz - 1) { c = L.cz[q + sz]; s += c * p[q + sz]; d += c; }
}

// (i, j, k) of cell q: shifts and masks for power-of-two levels
template <typename T>
__device__ __forceinline__ void sub_ijk(const SubLevel<T>& L, int q, int& i, int& j, int& k) {
  if (L.lx >= 0) {
    i = q & (L.nx - 1);
    j = (q >> L.lx) & (L.ny - 1);
    k = q >> (L.lx + L.ly);
  } else {
    i = q % L.nx;
    j = (q / L.nx) % L.ny;
    k = q / (L.nx * L.ny);
  }
}

// one colour of a red-black sweep on a shared-memory level: the threads walk
// the cells of the colour only (one per x pair of each row)
template <typename T>
__device__ void sub_colour(const SubLevel<T>& L, T* sol, const T* src, int color, bool zero) {
  const int hx = (L.nx + 1) >> 1;
  const int npair = hx * L.ny * L.nz;
  const bool shifts = L.lx >= 1;  // nx a power of two >= 2: hx = nx/2 = 2^(lx-1)
  for (int t = threadIdx.x; t < npair; t += blockDim.x) {
    int m, j, k;
    if (shifts) {
      m = t & (hx - 1);
      const int row = t >> (L.lx - 1);
      j = row & (L.ny - 1);
      k = row >> L.ly;
    } else {
      m = t % hx;
      const int row = t / hx;
      j = row % L.ny;
      k = row / L.ny;
    }
    const int i = 2 * m + ((j + k + color) & 1);
    if (i >= L.nx) continue;
    const int q = (k * L.ny + j) * L.nx + i;
    T s, d;
    if (zero) {
      T dd;
      sub_stencil(L, sol, i, j, k, q, s, dd);  // for d only; p is ignored
      s = T(0);
      d = dd;
    } else {
      sub_stencil(L, sol, i, j, k, q, s, d);
    }
    sol[q] = (s - src[q]) / d;
  }
  __syncthreads();
}

template <typename T>
__device__ void sub_sweep(const SubLevel<T>& L, T* sol, const T* src, int first, bool zero) {
  sub_colour(L, sol, src, first, zero);
  sub_colour(L, sol, src, 1 - first, false);
}

// coarse src = mean of the children's residuals (fine -> coarse, shared memory)
template <typename T>
__device__ void sub_restrict(const SubLevel<T>& F, const T* fsol, const T* fsrc,
                             const SubLevel<T>& C, T* csrc) {
  const int n = C.nx * C.ny * C.nz;
  for (int cq = threadIdx.x; cq < n; cq += blockDim.x) {
    int I, J, K;
    sub_ijk(C, cq, I, J, K);
    T acc = T(0);
    for (int dz = 0; dz < F.fz; ++dz)
      for (int dy = 0; dy < F.fy; ++dy)
        for (int dx = 0; dx < F.fx; ++dx) {
          const int i = F.fx * I + dx, j = F.fy * J + dy, k = F.fz * K + dz;
          const int q = (k * F.ny + j) * F.nx + i;
          T s, d;
          sub_stencil(F, fsol, i, j, k, q, s, d);
          acc += fsrc[q] - (s - d * fsol[q]);
        }
    csrc[cq] = acc * (T(1) / T(F.fx * F.fy * F.fz));
  }
  __syncthreads();
}

// fine sol += central-slope interpolation of the coarse sol
template <typename T>
__device__ void sub_prolong(const SubLevel<T>& F, T* fsol, const SubLevel<T>& C, const T* e) {
  const int n = F.nx * F.ny * F.nz;
  const int csy = C.nx, csz = C.nx * C.ny;
  for (int q = threadIdx.x; q < n; q += blockDim.x) {
    int i, j, k;
    sub_ijk(F, q, i, j, k);
    const int I = i >> (F.fx - 1), J = j >> (F.fy - 1), K = k >> (F.fz - 1);
    const int cq = K * csz + J * csy + I;
    const T ec = e[cq];
    T val = ec;
    if (F.fx == 2) {
      const T m = T(0.5) * ((I < C.nx - 1 ? e[cq + 1] : ec) - (I > 0 ? e[cq - 1] : ec));
      val += (i & 1) ? T(0.25) * m : -(T(0.25) * m);
    }
    if (F.fy == 2) {
      const T m = T(0.5) * ((J < C.ny - 1 ? e[cq + csy] : ec) - (J > 0 ? e[cq - csy] : ec));
      val += (j & 1) ? T(0.25) * m : -(T(0.25) * m);
    }
    if (F.fz == 2) {
      const T m = T(0.5) * ((K < C.nz - 1 ? e[cq + csz] : ec) - (K > 0 ? e[cq - csz] : ec));
      val += (k & 1) ? T(0.25) * m : -(T(0.25) * m);
    }
    fsol[q] += val;
  }
  __syncthreads();
}

// x = Minv b, one refinement step when max|b - A x| > 1e-10, mean projection
// (as k_coarse_solve)
template <typename T>
__device__ void sub_coarse(int n, const T* __restrict__ minv, const T* __restrict__ a, const T* b,
                           T* x, T* scratch) {
  T* se = scratch;           // n
  int* refine = reinterpret_cast<int*>(scratch + n);
  const int t = threadIdx.x;
  if (t == 0) *refine = 0;
  __syncthreads();
  if (t < n) {
    T acc = T(0);
    for (int q = 0; q < n; ++q) acc += minv[t * n + q] * b[q];
    x[t] = acc;
  }
  __syncthreads();
  if (t < n) {
    T e = b[t];
    for (int q = 0; q < n; ++q) e -= a[t * n + q] * x[q];
    se[t] = e;
    if (fabs((double)e) > 1e-10) atomicOr(refine, 1);
  }
  __syncthreads();
  if (*refine && t < n) {
    T acc = T(0);
    for (int q = 0; q < n; ++q) acc += minv[t * n + q] * se[q];
    x[t] += acc;
  }
  __syncthreads();
  if (t == 0) {
    T s = T(0);
    for (int q = 0; q < n; ++q) s += x[q];
    se[0] = s / T(n);
  }
  __syncthreads();
  if (t < n) x[t] -= se[0];
  __syncthreads();
}

// Shared memory per level: sol, src, then the three face-coefficient arrays
// (staged once at the start, so no phase waits on L2), n cells each.
template <typename T>
__device__ void subcycle_body(const SubCycle<T>& S, T* base) {
  const int nl = S.nlev;
  const auto cells = [&](int l) { return S.lv[l].nx * S.lv[l].ny * S.lv[l].nz; };
  const auto sol = [&](int l) { return base + S.off[l]; };
  const auto src = [&](int l) { return base + S.off[l] + cells(l); };
  for (int l = 0; l < nl; ++l) {
    const int n = cells(l);
    T* c = base + S.off[l] + 2 * n;
    for (int q = threadIdx.x; q < n; q += blockDim.x) {
      c[q] = S.lv[l].cx[q];
      c[n + q] = S.lv[l].cy[q];
      c[2 * n + q] = S.lv[l].cz[q];
    }
  }
  // level l with its coefficients in shared memory
  const auto lv = [&](int l) {
    SubLevel<T> L = S.lv[l];
    const int n = L.nx * L.ny * L.nz;
    const T* c = base + S.off[l] + 2 * n;
    L.cx = c;
    L.cy = c + n;
    L.cz = c + 2 * n;
    return L;
  };
  T* scratch = base + S.off[nl];
  {
    const int n0 = S.lv[0].nx * S.lv[0].ny * S.lv[0].nz;
    for (int q = threadIdx.x; q < n0; q += blockDim.x) src(0)[q] = __ldcg(S.src_in + q);
  }
  __syncthreads();
  for (int l = 0; l < nl - 1; ++l) {
    for (int it = 0; it < S.nu1; ++it) sub_sweep(lv(l), sol(l), src(l), 0, it == 0);
    if (S.nu1 == 0) {
      const int n = S.lv[l].nx * S.lv[l].ny * S.lv[l].nz;
      for (int q = threadIdx.x; q < n; q += blockDim.x) sol(l)[q] = T(0);
      __syncthreads();
    }
    sub_restrict(lv(l), sol(l), src(l), lv(l + 1), src(l + 1));
  }
  sub_coarse(S.n_coarse, S.minv, S.adense, src(nl - 1), sol(nl - 1), scratch);
  for (int l = nl - 2; l >= 0; --l) {
    sub_prolong(lv(l), sol(l), lv(l + 1), sol(l + 1));
    for (int it = 0; it < S.nu2; ++it) sub_sweep(lv(l), sol(l), src(l), S.reverse ? 1 : 0, false);
  }
  const int n0 = S.lv[0].nx * S.lv[0].ny * S.lv[0].nz;
  for (int q = threadIdx.x; q < n0; q += blockDim.x) S.sol_out[q] = sol(0)[q];
}

template <typename T>
__global__ void __launch_bounds__(kSubThreads) k_subcycle(SubCycle<T> S) {
  pdl_enter();
  extern __shared__ unsigned char sub_raw[];
  subcycle_body(S, reinterpret_cast<T*>(sub_raw));
}

// ---- the middle of the cycle: one cooperative launch ------------------------
// Levels between the finest and the single-block bottom (128^3 .. 32^3 for a
// 256^3 grid) take a few microseconds of work per sweep colour but one launch
// each, ~30 launches per cycle.  k_midcycle runs all their phases -- sweeps,
// residual + restriction, the bottom block (block 0 alone, in its shared
// memory), prolongation -- in one cooperative launch whose blocks are all
// resident, separated by a grid barrier.  Every phase calls the per-cell
// functions of the separate kernels (mg_cells.cuh), reading the unknowns past
// L1 because other blocks rewrite them between phases, so the cycle is the
// same cycle, bit for bit.
//
// The barrier is bounded: a block that waits more than kBarrierSpins polls
// sets kErrBarrierTimeout and the kernel returns (every other block then
// times out at its next barrier), so a fault of the co-residency assumption
// can only end the launch, never hang it.
constexpr unsigned kBarrierSpins = 1u << 22;
constexpr int kErrBarrierTimeout = 2;

__device__ __forceinline__ bool grid_barrier(unsigned* bar, int* err) {
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned* gen = bar + 1;
    const unsigned g = *gen;
    int good = 1;
    __threadfence();
    if (atomicAdd(bar, 1u) + 1u == gridDim.x) {
      atomicExch(bar, 0u);
      __threadfence();
      atomicAdd(bar + 1, 1u);
    } else {
      unsigned spins = 0;
      while (*gen == g) {
        if (++spins > kBarrierSpins) {
          atomicOr(err, kErrBarrierTimeout);
          good = 0;
          break;
        }
        __nanosleep(32);
      }
    }
    __threadfence();
    ok = good;
  }
  __syncthreads();
  return ok != 0;
}

template <typename T>
__device__ __forceinline__ void mid_colour(const LevelView<T>& L, int color, bool zero) {
  const int hx = (L.nx + 1) / 2;
  const size_t n = (size_t)hx * L.ny * L.nz;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += stride) {
    const int m = (int)(t % hx);
    const size_t row = t / hx;
    const int j = (int)(row % L.ny), k = (int)(row / L.ny);
    const int i = 2 * m + ((j + k + color) & 1);
    if (i >= L.nx) continue;
    if (L.idiag) {
      if (zero) cells::smooth_cell<T, true, true, false, true>(L, i, j, k);
      else cells::smooth_cell<T, true, false, false, true>(L, i, j, k);
    } else {
      if (zero) cells::smooth_cell<T, false, true, false, true>(L, i, j, k);
      else cells::smooth_cell<T, false, false, false, true>(L, i, j, k);
    }
  }
}

template <typename T>
__device__ __forceinline__ void mid_restrict(const LevelView<T>& F, const LevelView<T>& C,
                                             int zero_sol) {
  const size_t n = (size_t)C.nx * C.ny * C.nz;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += stride) {
    const int I = (int)(t % C.nx);
    const size_t row = t / C.nx;
    cells::restrict_cell<T, false, true>(F, C, I, (int)(row % C.ny), (int)(row / C.ny), zero_sol);
  }
}

template <typename T>
__device__ __forceinline__ void mid_prolong(const LevelView<T>& F, const LevelView<T>& C) {
  const size_t n = (size_t)C.nx * C.ny * C.nz;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += stride) {
    const int I = (int)(t % C.nx);
    const size_t row = t / C.nx;
    cells::prolong_cell<T, true>(F, C, I, (int)(row % C.ny), (int)(row / C.ny));
  }
}

template <typename T>
__global__ void __launch_bounds__(kMidThreads) k_midcycle(MidCycle<T> M) {
  extern __shared__ unsigned char mid_raw[];
  T* base = reinterpret_cast<T*>(mid_raw);
  const int nm = M.nmid;
  // down: levels 0 .. nm-1 of M.lv are the middle levels, M.lv[nm] the bottom's top
  for (int l = 0; l < nm; ++l) {
    for (int it = 0; it < M.nu1; ++it) {
      mid_colour(M.lv[l], 0, it == 0);
      if (!grid_barrier(M.bar, M.err)) return;
      mid_colour(M.lv[l], 1, false);
      if (!grid_barrier(M.bar, M.err)) return;
    }
    mid_restrict(M.lv[l], M.lv[l + 1], M.nu1 > 0 ? 0 : 1);
    if (!grid_barrier(M.bar, M.err)) return;
  }
  if (blockIdx.x == 0) subcycle_body(M.bottom, base);
  if (!grid_barrier(M.bar, M.err)) return;
  const int c0 = M.reverse ? 1 : 0;
  for (int l = nm - 1; l >= 0; --l) {
    mid_prolong(M.lv[l], M.lv[l + 1]);
    if (!grid_barrier(M.bar, M.err)) return;
    for (int it = 0; it < M.nu2; ++it) {
      mid_colour(M.lv[l], c0, false);
      if (!grid_barrier(M.bar, M.err)) return;
      mid_colour(M.lv[l], 1 - c0, false);
      if (l > 0 || it + 1 < M.nu2)  // the last phase ends with the kernel
        if (!grid_barrier(M.bar, M.err)) return;
    }
  }
}

}  // namespace

template <typename T>
size_t subcycle_smem(const SubCycle<T>& S) {
  return (size_t)(S.off[S.nlev] + 2 * kMaxCoarse + 8) * sizeof(T);
}

template <typename T>
int subcycle_init(size_t smem) {
  return cudaFuncSetAttribute(k_subcycle<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)smem) == cudaSuccess
             ? 0
             : -1;
}

template <typename T>
void launch_subcycle(cudaStream_t s, const SubCycle<T>& S) {
  launch_pdl(k_subcycle<T>, dim3(1), dim3(kSubThreads), subcycle_smem(S), s, S);
}

template size_t subcycle_smem<float>(const SubCycle<float>&);
template size_t subcycle_smem<double>(const SubCycle<double>&);
template int subcycle_init<float>(size_t);
template int subcycle_init<double>(size_t);
template void launch_subcycle<float>(cudaStream_t, const SubCycle<float>&);
template void launch_subcycle<double>(cudaStream_t, const SubCycle<double>&);

template <typename T>
size_t midcycle_smem(const MidCycle<T>& M) {
  return subcycle_smem(M.bottom);  // block 0 runs the bottom in its shared memory
}

template <typename T>
int midcycle_init(size_t smem, int* grid_blocks) {
  if (cudaFuncSetAttribute(k_midcycle<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)smem) != cudaSuccess)
    return -1;
  int per_sm = 0, dev = 0, sms = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_midcycle<T>, kMidThreads, smem) !=
          cudaSuccess ||
      per_sm < 1)
    return -1;
  cudaGetDevice(&dev);
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return -1;
  *grid_blocks = per_sm * sms;
  return 0;
}

template <typename T>
cudaError_t launch_midcycle(cudaStream_t s, const MidCycle<T>& M, int grid_blocks) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)grid_blocks);
  cfg.blockDim = dim3(kMidThreads);
  cfg.dynamicSmemBytes = midcycle_smem(M);
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, k_midcycle<T>, M);
}

template size_t midcycle_smem<float>(const MidCycle<float>&);
template size_t midcycle_smem<double>(const MidCycle<double>&);
template int midcycle_init<float>(size_t, int*);
template int midcycle_init<double>(size_t, int*);
template cudaError_t launch_midcycle<float>(cudaStream_t, const MidCycle<float>&, int);
template cudaError_t launch_midcycle<double>(cudaStream_t, const MidCycle<double>&, int);

}  // namespace gbmg
