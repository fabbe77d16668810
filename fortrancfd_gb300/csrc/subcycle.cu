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

// ---- the bottom of the cycle on a thread-block cluster ----------------------
// The same cycle as k_subcycle from a larger first level (up to
// kClusterMaxCells cells, 32^3), on the P.ranks blocks of one cluster, one
// per SM.  The finer levels are split by z planes: block r holds planes
// [r*pz, min(nz, (r+1)*pz)) of sol, src and the three coefficient arrays in
// its shared memory and reads the planes of other blocks through distributed
// shared memory (mapa addresses).  A sweep colour updates the block's own
// cells; only the z neighbours across a slab edge are remote.  Restriction is
// computed by the block that holds the children (or, when slabs do not align
// with the children, by the one that holds the coarse cell), prolongation by
// the block that holds the fine cell.  The coarsest levels ("single") lie
// whole in block 0, which runs them as k_subcycle does, with __syncthreads
// between phases, while the other blocks wait at the next cluster barrier.
// Phases of split levels end in a hardware cluster barrier
// (barrier.cluster arrive.release / wait.acquire), which every thread of
// every block reaches the same number of times, so it needs no spin of its
// own.  The arithmetic of each cell is that of sub_colour / sub_restrict /
// sub_prolong / sub_coarse, in the same order.
__device__ __forceinline__ unsigned cl_rank() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}

__device__ __forceinline__ void cl_sync() {
  asm volatile(
      "barrier.cluster.arrive.release.aligned;\n\t"
      "barrier.cluster.wait.acquire.aligned;" ::: "memory");
}

template <typename T>
__device__ __forceinline__ T* cl_map(T* p, unsigned r) {
  unsigned long long out;
  asm volatile("mapa.u64 %0, %1, %2;" : "=l"(out) : "l"(p), "r"(r));
  return reinterpret_cast<T*>(out);
}

// array a (0 sol, 1 src, 2 cx, 3 cy, 4 cz) of cell (i, j, k) of level l, in
// the block that holds plane k
template <typename T>
__device__ __forceinline__ T& cl_at(const ClusterCycle<T>& P, T* const* rb, int l, int a, int i,
                                    int j, int k) {
  const SubLevel<T>& L = P.S.lv[l];
  const int pz = P.pz[l];
  const int r = P.lpz[l] >= 0 ? (k >> P.lpz[l]) : k / pz;
  const int kk = k - r * pz;
  return rb[r][P.off[l] + a * pz * L.nx * L.ny + (kk * L.ny + j) * L.nx + i];
}

// sub_stencil of any cell, every value read from the block that holds it
template <typename T>
__device__ __forceinline__ void cl_stencil(const ClusterCycle<T>& P, T* const* rb, int l, int i,
                                           int j, int k, T& s, T& d) {
  const SubLevel<T>& L = P.S.lv[l];
  T c;
  s = T(0);
  d = T(0);
  if (i > 0) { c = cl_at(P, rb, l, 2, i, j, k); s += c * cl_at(P, rb, l, 0, i - 1, j, k); d += c; }
  if (i < L.nx - 1) { c = cl_at(P, rb, l, 2, i + 1, j, k); s += c * cl_at(P, rb, l, 0, i + 1, j, k); d += c; }
  if (j > 0) { c = cl_at(P, rb, l, 3, i, j, k); s += c * cl_at(P, rb, l, 0, i, j - 1, k); d += c; }
  if (j < L.ny - 1) { c = cl_at(P, rb, l, 3, i, j + 1, k); s += c * cl_at(P, rb, l, 0, i, j + 1, k); d += c; }
  if (k > 0) { c = cl_at(P, rb, l, 4, i, j, k); s += c * cl_at(P, rb, l, 0, i, j, k - 1); d += c; }
  if (k < L.nz - 1) { c = cl_at(P, rb, l, 4, i, j, k + 1); s += c * cl_at(P, rb, l, 0, i, j, k + 1); d += c; }
}

// sub_stencil of a cell of the block's own planes (local index q, local plane
// kk): everything from the block's shared memory except the z neighbour
// across a slab edge; zero: p taken as 0 (s stays 0)
template <typename T>
__device__ __forceinline__ void cl_own_stencil(const ClusterCycle<T>& P, T* const* rb, int l,
                                               const T* sol, int q, int i, int j, int k, int kk,
                                               bool zero, T& s, T& d) {
  const SubLevel<T>& L = P.S.lv[l];
  const int nx = L.nx, pz = P.pz[l], plane = nx * L.ny, cap = pz * plane;
  const T* cx = sol + 2 * cap;
  const T* cy = sol + 3 * cap;
  const T* cz = sol + 4 * cap;
  T c;
  s = T(0);
  d = T(0);
  if (i > 0) { c = cx[q]; if (!zero) s += c * sol[q - 1]; d += c; }
  if (i < nx - 1) { c = cx[q + 1]; if (!zero) s += c * sol[q + 1]; d += c; }
  if (j > 0) { c = cy[q]; if (!zero) s += c * sol[q - nx]; d += c; }
  if (j < L.ny - 1) { c = cy[q + nx]; if (!zero) s += c * sol[q + nx]; d += c; }
  if (k > 0) {
    c = cz[q];
    if (!zero) s += c * (kk > 0 ? sol[q - plane] : cl_at(P, rb, l, 0, i, j, k - 1));
    d += c;
  }
  if (k < L.nz - 1) {
    const bool own = kk + 1 < pz;
    c = own ? cz[q + plane] : cl_at(P, rb, l, 4, i, j, k + 1);
    if (!zero) s += c * (own ? sol[q + plane] : cl_at(P, rb, l, 0, i, j, k + 1));
    d += c;
  }
}

// one colour on the block's own planes (sub_colour)
template <typename T>
__device__ void cl_colour(const ClusterCycle<T>& P, T* raw, T* const* rb, int me, int l,
                          int color, bool zero) {
  const SubLevel<T>& L = P.S.lv[l];
  const int nx = L.nx, ny = L.ny, nz = L.nz, pz = P.pz[l];
  const int cap = pz * nx * ny;
  const int k0 = me * pz, k1 = min(nz, k0 + pz);
  T* sol = raw + P.off[l];
  const T* src = sol + cap;
  const int hx = (nx + 1) >> 1;
  const int npair = k1 > k0 ? hx * ny * (k1 - k0) : 0;
  const bool shifts = L.lx >= 1;  // nx a power of two >= 2: hx = 2^(lx-1)
  for (int t = threadIdx.x; t < npair; t += blockDim.x) {
    int m, j, kk;
    if (shifts) {
      m = t & (hx - 1);
      const int row = t >> (L.lx - 1);
      j = row & (ny - 1);
      kk = row >> L.ly;
    } else {
      m = t % hx;
      const int row = t / hx;
      j = row % ny;
      kk = row / ny;
    }
    const int k = k0 + kk;
    const int i = 2 * m + ((j + k + color) & 1);
    if (i >= nx) continue;
    const int q = (kk * ny + j) * nx + i;
    T s, d;
    cl_own_stencil(P, rb, l, sol, q, i, j, k, kk, zero, s, d);
    sol[q] = (s - src[q]) / d;
  }
  cl_sync();
}

// coarse src = mean of the children's residuals (sub_restrict).  When every
// block's slab starts on a child boundary (pz % fz == 0) the block that holds
// the children computes the coarse cell (written to whichever block holds
// it: block 0 for a single coarse level); otherwise the block that holds the
// coarse cell computes it from children read wherever they are.
template <typename T>
__device__ void cl_restrict(const ClusterCycle<T>& P, T* raw, T* const* rb, int me, int l) {
  const SubLevel<T>& F = P.S.lv[l];
  const SubLevel<T>& C = P.S.lv[l + 1];
  const int cplane = C.nx * C.ny;
  const T scale = T(1) / T(F.fx * F.fy * F.fz);
  const int pzf = P.pz[l];
  if (pzf % F.fz == 0) {
    const int capf = pzf * F.nx * F.ny, k0f = me * pzf, k1f = min(F.nz, k0f + pzf);
    const int K0 = k0f / F.fz;
    const int n = k1f > k0f ? ((k1f - k0f) / F.fz) * cplane : 0;
    const T* fsol = raw + P.off[l];
    const T* fsrc = fsol + capf;
    for (int t = threadIdx.x; t < n; t += blockDim.x) {
      int I, J, KK;
      sub_ijk(C, t, I, J, KK);
      T acc = T(0);
      for (int dz = 0; dz < F.fz; ++dz)
        for (int dy = 0; dy < F.fy; ++dy)
          for (int dx = 0; dx < F.fx; ++dx) {
            const int i = F.fx * I + dx, j = F.fy * J + dy, kk = F.fz * KK + dz;
            const int q = (kk * F.ny + j) * F.nx + i;
            T s, d;
            cl_own_stencil(P, rb, l, fsol, q, i, j, k0f + kk, kk, false, s, d);
            acc += fsrc[q] - (s - d * fsol[q]);
          }
      cl_at(P, rb, l + 1, 1, I, J, K0 + KK) = acc * scale;
    }
  } else {
    const int pz = P.pz[l + 1];
    const int k0 = me * pz, k1 = min(C.nz, k0 + pz);
    const int n = k1 > k0 ? (k1 - k0) * cplane : 0;
    for (int t = threadIdx.x; t < n; t += blockDim.x) {
      const int I = t % C.nx, J = (t / C.nx) % C.ny, K = k0 + t / cplane;
      T acc = T(0);
      for (int dz = 0; dz < F.fz; ++dz)
        for (int dy = 0; dy < F.fy; ++dy)
          for (int dx = 0; dx < F.fx; ++dx) {
            const int i = F.fx * I + dx, j = F.fy * J + dy, k = F.fz * K + dz;
            T s, d;
            cl_stencil(P, rb, l, i, j, k, s, d);
            acc += cl_at(P, rb, l, 1, i, j, k) - (s - d * cl_at(P, rb, l, 0, i, j, k));
          }
      cl_at(P, rb, l + 1, 1, I, J, K) = acc * scale;
    }
  }
  cl_sync();
}

// the block's own fine cells += central-slope interpolation (sub_prolong);
// the parents are local when the block's coarse planes are exactly the
// parents of its fine planes
template <typename T>
__device__ void cl_prolong(const ClusterCycle<T>& P, T* raw, T* const* rb, int me, int l) {
  const SubLevel<T>& F = P.S.lv[l];
  const SubLevel<T>& C = P.S.lv[l + 1];
  const int pz = P.pz[l], plane = F.nx * F.ny;
  const int k0 = me * pz, k1 = min(F.nz, k0 + pz);
  T* fsol = raw + P.off[l];
  const int n = k1 > k0 ? (k1 - k0) * plane : 0;
  const int pzc = P.pz[l + 1], cplane = C.nx * C.ny;
  const bool local = pz == F.fz * pzc;
  const T* e = raw + P.off[l + 1];
  for (int q = threadIdx.x; q < n; q += blockDim.x) {
    int i, j, kk;
    sub_ijk(F, q, i, j, kk);
    const int k = k0 + kk;
    const int I = i >> (F.fx - 1), J = j >> (F.fy - 1), K = k >> (F.fz - 1);
    T ec, exm, exp_, eym, eyp, ezm, ezp;
    if (local) {
      const int KK = kk >> (F.fz - 1);
      const int cq = (KK * C.ny + J) * C.nx + I;
      ec = e[cq];
      exp_ = I < C.nx - 1 ? e[cq + 1] : ec;
      exm = I > 0 ? e[cq - 1] : ec;
      eyp = J < C.ny - 1 ? e[cq + C.nx] : ec;
      eym = J > 0 ? e[cq - C.nx] : ec;
      ezp = K < C.nz - 1 ? (KK + 1 < pzc ? e[cq + cplane] : cl_at(P, rb, l + 1, 0, I, J, K + 1)) : ec;
      ezm = K > 0 ? (KK > 0 ? e[cq - cplane] : cl_at(P, rb, l + 1, 0, I, J, K - 1)) : ec;
    } else {
      ec = cl_at(P, rb, l + 1, 0, I, J, K);
      exp_ = I < C.nx - 1 ? cl_at(P, rb, l + 1, 0, I + 1, J, K) : ec;
      exm = I > 0 ? cl_at(P, rb, l + 1, 0, I - 1, J, K) : ec;
      eyp = J < C.ny - 1 ? cl_at(P, rb, l + 1, 0, I, J + 1, K) : ec;
      eym = J > 0 ? cl_at(P, rb, l + 1, 0, I, J - 1, K) : ec;
      ezp = K < C.nz - 1 ? cl_at(P, rb, l + 1, 0, I, J, K + 1) : ec;
      ezm = K > 0 ? cl_at(P, rb, l + 1, 0, I, J, K - 1) : ec;
    }
    T val = ec;
    if (F.fx == 2) {
      const T m = T(0.5) * (exp_ - exm);
      val += (i & 1) ? T(0.25) * m : -(T(0.25) * m);
    }
    if (F.fy == 2) {
      const T m = T(0.5) * (eyp - eym);
      val += (j & 1) ? T(0.25) * m : -(T(0.25) * m);
    }
    if (F.fz == 2) {
      const T m = T(0.5) * (ezp - ezm);
      val += (k & 1) ? T(0.25) * m : -(T(0.25) * m);
    }
    fsol[q] += val;
  }
  cl_sync();
}

template <typename T>
__global__ void __launch_bounds__(kSubThreads) k_cluster_cycle(ClusterCycle<T> P) {
  pdl_enter();
  extern __shared__ unsigned char cl_raw[];
  T* raw = reinterpret_cast<T*>(cl_raw);
  __shared__ T* rb[kClusterMaxRanks];
  const int me = (int)cl_rank();
  const SubCycle<T>& S = P.S;
  const int nl = S.nlev, ns = P.nsplit;
  if (threadIdx.x < P.ranks) rb[threadIdx.x] = cl_map(raw, threadIdx.x);
  // stage the own planes of every level's coefficients (single levels: block
  // 0) and of the first level's right-hand side
  for (int l = 0; l < nl; ++l) {
    const SubLevel<T>& L = S.lv[l];
    const int pz = P.pz[l], plane = L.nx * L.ny, cap = pz * plane;
    const int k0 = me * pz, k1 = min(L.nz, k0 + pz);
    const int n = k1 > k0 ? (k1 - k0) * plane : 0;
    const size_t g0 = (size_t)k0 * plane;
    T* c = raw + P.off[l] + 2 * cap;
    for (int q = threadIdx.x; q < n; q += blockDim.x) {
      c[q] = L.cx[g0 + q];
      c[cap + q] = L.cy[g0 + q];
      c[2 * cap + q] = L.cz[g0 + q];
    }
    if (l == 0)
      for (int q = threadIdx.x; q < n; q += blockDim.x)
        raw[P.off[0] + cap + q] = __ldcg(S.src_in + g0 + q);
  }
  cl_sync();  // every block has started and staged its planes
  const int top = min(ns, nl - 1);  // split levels with a coarser level below
  for (int l = 0; l < top; ++l) {
    for (int it = 0; it < S.nu1; ++it) {
      cl_colour(P, raw, rb, me, l, 0, it == 0);
      cl_colour(P, raw, rb, me, l, 1, false);
    }
    if (S.nu1 == 0) {
      const SubLevel<T>& L = S.lv[l];
      const int pz = P.pz[l], plane = L.nx * L.ny;
      for (int q = threadIdx.x; q < pz * plane; q += blockDim.x) raw[P.off[l] + q] = T(0);
      cl_sync();
    }
    cl_restrict(P, raw, rb, me, l);
  }
  if (ns < nl) {
    // the single levels, whole in block 0, as in subcycle_body
    if (me == 0) {
      const auto cells = [&](int l) { return S.lv[l].nx * S.lv[l].ny * S.lv[l].nz; };
      const auto sol = [&](int l) { return raw + P.off[l]; };
      const auto src = [&](int l) { return raw + P.off[l] + cells(l); };
      const auto lv = [&](int l) {
        SubLevel<T> L = S.lv[l];
        const int n = cells(l);
        const T* c = raw + P.off[l] + 2 * n;
        L.cx = c;
        L.cy = c + n;
        L.cz = c + 2 * n;
        return L;
      };
      for (int l = ns; l < nl - 1; ++l) {
        for (int it = 0; it < S.nu1; ++it) sub_sweep(lv(l), sol(l), src(l), 0, it == 0);
        if (S.nu1 == 0) {
          for (int q = threadIdx.x; q < cells(l); q += blockDim.x) sol(l)[q] = T(0);
          __syncthreads();
        }
        sub_restrict(lv(l), sol(l), src(l), lv(l + 1), src(l + 1));
      }
      sub_coarse(S.n_coarse, S.minv, S.adense, src(nl - 1), sol(nl - 1), raw + P.off[nl]);
      for (int l = nl - 2; l >= ns; --l) {
        sub_prolong(lv(l), sol(l), lv(l + 1), sol(l + 1));
        for (int it = 0; it < S.nu2; ++it) sub_sweep(lv(l), sol(l), src(l), S.reverse ? 1 : 0, false);
      }
    }
    cl_sync();
  } else {
    // the coarsest level is split: gathered into block 0 (sub_coarse)
    const SubLevel<T>& L = S.lv[nl - 1];
    const int n = S.n_coarse;
    if (me == 0) {
      T* gb = raw + P.off[nl];
      T* gx = gb + n;
      for (int q = threadIdx.x; q < n; q += blockDim.x)
        gb[q] = cl_at(P, rb, nl - 1, 1, q % L.nx, (q / L.nx) % L.ny, q / (L.nx * L.ny));
      __syncthreads();
      sub_coarse(n, S.minv, S.adense, gb, gx, gx + n);
      for (int q = threadIdx.x; q < n; q += blockDim.x)
        cl_at(P, rb, nl - 1, 0, q % L.nx, (q / L.nx) % L.ny, q / (L.nx * L.ny)) = gx[q];
    }
    cl_sync();
  }
  for (int l = top - 1; l >= 0; --l) {
    cl_prolong(P, raw, rb, me, l);
    const int c0 = S.reverse ? 1 : 0;
    for (int it = 0; it < S.nu2; ++it) {
      cl_colour(P, raw, rb, me, l, c0, false);
      cl_colour(P, raw, rb, me, l, 1 - c0, false);
    }
  }
  {
    const SubLevel<T>& L = S.lv[0];
    const int pz = P.pz[0], plane = L.nx * L.ny;
    const int k0 = me * pz, k1 = min(L.nz, k0 + pz);
    const int n = k1 > k0 ? (k1 - k0) * plane : 0;
    for (int q = threadIdx.x; q < n; q += blockDim.x)
      S.sol_out[(size_t)k0 * plane + q] = raw[P.off[0] + q];
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
ClusterCycle<T> make_cluster_cycle(const SubCycle<T>& S, int ranks, int single_cells) {
  ClusterCycle<T> P{};
  P.S = S;
  P.ranks = ranks;
  P.nsplit = S.nlev;
  int off = 0;
  for (int l = 0; l < S.nlev; ++l) {
    const SubLevel<T>& L = S.lv[l];
    const bool single = l > 0 && L.nx * L.ny * L.nz <= single_cells;
    if (single && P.nsplit == S.nlev) P.nsplit = l;
    P.pz[l] = l >= P.nsplit ? L.nz : (L.nz + ranks - 1) / ranks;
    P.lpz[l] = -1;
    for (int b = 0; b < 31; ++b)
      if ((1 << b) == P.pz[l]) P.lpz[l] = b;
    P.off[l] = off;
    off += 5 * P.pz[l] * L.nx * L.ny;  // sol, src, cx, cy, cz of the block's planes
  }
  P.off[S.nlev] = off;  // block 0: coarse gather (b, x) and the solve's scratch
  return P;
}

template <typename T>
size_t cluster_smem(const ClusterCycle<T>& P) {
  return (size_t)(P.off[P.S.nlev] + 3 * kMaxCoarse + 8) * sizeof(T);
}

template <typename T>
int cluster_init(size_t smem, int ranks) {
  if (ranks < 1 || ranks > kClusterMaxRanks) return -1;
  if (cudaFuncSetAttribute(k_cluster_cycle<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)smem) != cudaSuccess)
    return -1;
  if (ranks > 8 &&
      cudaFuncSetAttribute(k_cluster_cycle<T>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) !=
          cudaSuccess) {
    cudaGetLastError();
    return -1;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(ranks);
  cfg.blockDim = dim3(kSubThreads);
  cfg.dynamicSmemBytes = smem;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = ranks;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  int clusters = 0;
  if (cudaOccupancyMaxActiveClusters(&clusters, k_cluster_cycle<T>, &cfg) != cudaSuccess ||
      clusters < 1) {
    cudaGetLastError();
    return -1;
  }
  return 0;
}

template <typename T>
cudaError_t launch_cluster_cycle(cudaStream_t s, const ClusterCycle<T>& P) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(P.ranks);
  cfg.blockDim = dim3(kSubThreads);
  cfg.dynamicSmemBytes = cluster_smem(P);
  cfg.stream = s;
  cudaLaunchAttribute at[2];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = P.ranks;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  at[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[1].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 2;
  return cudaLaunchKernelEx(&cfg, k_cluster_cycle<T>, P);
}

template ClusterCycle<float> make_cluster_cycle<float>(const SubCycle<float>&, int, int);
template ClusterCycle<double> make_cluster_cycle<double>(const SubCycle<double>&, int, int);
template size_t cluster_smem<float>(const ClusterCycle<float>&);
template size_t cluster_smem<double>(const ClusterCycle<double>&);
template int cluster_init<float>(size_t, int);
template int cluster_init<double>(size_t, int);
template cudaError_t launch_cluster_cycle<float>(cudaStream_t, const ClusterCycle<float>&);
template cudaError_t launch_cluster_cycle<double>(cudaStream_t, const ClusterCycle<double>&);

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
