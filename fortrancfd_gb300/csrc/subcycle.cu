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

}  // namespace gbmg
