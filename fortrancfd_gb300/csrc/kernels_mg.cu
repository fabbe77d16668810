// Multigrid kernels for sm_103a: red-black Gauss-Seidel smoother, fused
// residual + restriction, central-slope prolongation, fine-level residual
// norm, coarse-operator construction and the dense coarsest-level solve.
//
// The cycle restated here is the reference's ("DomainDecomposition/3D/src/
// others/multigrid_solver.f90": multigrid_relax :1-49, multigrid_restriction
// :51-90, multigrid_final_exact :92-104, multigrid_prolongation :106-160,
// multigrid_residual :162-222) applied to the variable-coefficient operator of
// ppe_sor_init ("Two phase flows/newOpenMP/3D+IBM/src/ns_solver/
// ns_ppe_solver.f90:1-65").  Operator: (A p)_i = sum_f coe_f (p_nb - p_i), with
// zero coefficients on walls.
#include <algorithm>
#include <cstdio>
#include <type_traits>

#include "gbmg_internal.h"
#include "pdl.cuh"
#include "reduce.cuh"

namespace gbmg {

namespace {

inline unsigned cdiv(size_t a, unsigned b) { return (unsigned)((a + b - 1) / b); }

// Neighbour sum s = sum_f coe_f p_nb and diagonal d = sum_f coe_f of cell
// (i,j,k), accumulated in the order x-, x+, y-, y+, z-, z+.
template <typename T>
__device__ __forceinline__ void stencil(const LevelView<T>& L, const T* __restrict__ p, int i,
                                        int j, int k, size_t q, T& s, T& d) {
  const size_t sy = (size_t)L.nx, sz = (size_t)L.nx * L.ny;
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

// Face coefficient k/(rho_a + rho_b) of the density form.  FP32 uses the
// approximate reciprocal (within 1 ulp): these coefficients only drive the
// FP32 smoother and restriction of the mixed-precision cycle, whose result is
// corrected against the FP64 operator.
template <typename T>
__device__ __forceinline__ T rho_face(T k, T ra, T rb) {
  if constexpr (std::is_same<T, float>::value) return rho_face32(k, ra, rb);
  else return k / (ra + rb);
}

// The density-form smoother's update (s - b)/d, with the approximate
// reciprocal (only the FP32 preconditioner uses it).
template <typename T>
__device__ __forceinline__ T rho_update(T v, T d) {
  if constexpr (std::is_same<T, float>::value) return rho_update32(v, d);
  else return v / d;
}

// stencil() with the coefficients computed from the density (same order).
template <typename T>
__device__ __forceinline__ void stencil_rho(const LevelView<T>& L, const T* __restrict__ p, int i,
                                            int j, int k, size_t q, T& s, T& d) {
  const size_t sy = (size_t)L.nx, sz = (size_t)L.nx * L.ny;
  const T* __restrict__ r = L.rho;
  const T rc = r[q];
  T c;
  s = T(0);
  d = T(0);
  if (i > 0) { c = rho_face(L.kx, rc, r[q - 1]); s += c * p[q - 1]; d += c; }
  if (i < L.nx - 1) { c = rho_face(L.kx, rc, r[q + 1]); s += c * p[q + 1]; d += c; }
  if (j > 0) { c = rho_face(L.ky, rc, r[q - sy]); s += c * p[q - sy]; d += c; }
  if (j < L.ny - 1) { c = rho_face(L.ky, rc, r[q + sy]); s += c * p[q + sy]; d += c; }
  if (k > 0) { c = rho_face(L.kz, rc, r[q - sz]); s += c * p[q - sz]; d += c; }
  if (k < L.nz - 1) { c = rho_face(L.kz, rc, r[q + sz]); s += c * p[q + sz]; d += c; }
}

// The diagonal sum_f coe_f alone (same order as stencil_rho).
template <typename T>
__device__ __forceinline__ T diag_rho(const LevelView<T>& L, int i, int j, int k, size_t q) {
  const size_t sy = (size_t)L.nx, sz = (size_t)L.nx * L.ny;
  const T* __restrict__ r = L.rho;
  const T rc = r[q];
  T d = T(0);
  if (i > 0) d += rho_face(L.kx, rc, r[q - 1]);
  if (i < L.nx - 1) d += rho_face(L.kx, rc, r[q + 1]);
  if (j > 0) d += rho_face(L.ky, rc, r[q - sy]);
  if (j < L.ny - 1) d += rho_face(L.ky, rc, r[q + sy]);
  if (k > 0) d += rho_face(L.kz, rc, r[q - sz]);
  if (k < L.nz - 1) d += rho_face(L.kz, rc, r[q + sz]);
  return d;
}

// Flux sum sum_f coe_f (p_nb - p_i) of cell (i,j,k), differences first so the
// rounding is relative to each flux rather than to d |p| (order x-, x+, y-,
// y+, z-, z+).
template <typename T>
__device__ __forceinline__ T flux_sum(const LevelView<T>& L, const T* __restrict__ p, int i, int j,
                                      int k, size_t q) {
  const size_t sy = (size_t)L.nx, sz = (size_t)L.nx * L.ny;
  const T pc = p[q];
  T s = T(0);
  if (i > 0) s += L.cx[q] * (p[q - 1] - pc);
  if (i < L.nx - 1) s += L.cx[q + 1] * (p[q + 1] - pc);
  if (j > 0) s += L.cy[q] * (p[q - sy] - pc);
  if (j < L.ny - 1) s += L.cy[q + sy] * (p[q + sy] - pc);
  if (k > 0) s += L.cz[q] * (p[q - sz] - pc);
  if (k < L.nz - 1) s += L.cz[q + sz] * (p[q + sz] - pc);
  return s;
}

// One colour of a red-black Gauss-Seidel sweep: cells with (i+j+k)%2 == color
// get p_i = (s - b_i)/d (the reference's p_i = (src - sum coe p_nb)/c with
// c = -d).  One thread per cell of the colour.
// kZero: the level's current values are taken as zero (the first colour of
// the first sweep from a zero initial guess), so p_i = -b_i/d and p is not read.
// kRho: coefficients from the density (stencil_rho).
template <typename T, bool kIdiag, bool kZero, bool kRho>
__global__ void __launch_bounds__(256) k_smooth(LevelView<T> L, int color) {
  pdl_enter();
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (j >= L.ny) return;
  const int i = 2 * (blockIdx.x * blockDim.x + threadIdx.x) + ((j + k + color) & 1);
  if (i >= L.nx) return;
  const size_t q = ((size_t)k * L.ny + j) * L.nx + i;
  T s, d;
  if (kRho) {
    if (kZero) {
      s = T(0);
      d = diag_rho(L, i, j, k, q);
    } else {
      stencil_rho(L, L.sol, i, j, k, q, s, d);
    }
  } else if (kZero) {
    const size_t sy = (size_t)L.nx, sz = (size_t)L.nx * L.ny;
    s = T(0);
    d = T(0);
    if (i > 0) d += L.cx[q];
    if (i < L.nx - 1) d += L.cx[q + 1];
    if (j > 0) d += L.cy[q];
    if (j < L.ny - 1) d += L.cy[q + sy];
    if (k > 0) d += L.cz[q];
    if (k < L.nz - 1) d += L.cz[q + sz];
  } else {
    stencil(L, L.sol, i, j, k, q, s, d);
  }
  const T v = s - L.src[q];
  if (kIdiag) L.sol[q] = v * L.idiag[q];
  else if (kRho) L.sol[q] = rho_update(v, d);
  else L.sol[q] = v / d;
}

template <typename T> struct Vec2;
template <> struct Vec2<float> { using type = float2; };
template <> struct Vec2<double> { using type = double2; };

// Fused residual + restriction: coarse src = mean over the children of
// (src - A sol) on the fine level; coarse sol = 0.  One thread per coarse
// cell; the children are summed in the order z, y, x (the oracle's).
template <typename T, bool kRho>
__global__ void __launch_bounds__(256) k_restrict(LevelView<T> F, LevelView<T> C, int zero_sol) {
  pdl_enter();
  const int I = blockIdx.x * blockDim.x + threadIdx.x;
  const int J = blockIdx.y * blockDim.y + threadIdx.y;
  const int K = blockIdx.z;
  if (I >= C.nx || J >= C.ny) return;
  T acc = T(0);
  if (F.fx == 2) {
    // the two x-children of each child row as vector loads
    using V2 = typename Vec2<T>::type;
    const size_t sy = (size_t)F.nx, sz = (size_t)F.nx * F.ny;
    const int i0 = 2 * I;
    const V2 zero2{T(0), T(0)};
    for (int dz = 0; dz < F.fz; ++dz)
      for (int dy = 0; dy < F.fy; ++dy) {
        const int j = F.fy * J + dy, k = F.fz * K + dz;
        const size_t q = ((size_t)k * F.ny + j) * F.nx + i0;
        const V2 p = *reinterpret_cast<const V2*>(F.sol + q);
        const V2 b = *reinterpret_cast<const V2*>(F.src + q);
        const bool xl = i0 > 0, xr = i0 + 2 < F.nx;
        const bool yl = j > 0, yr = j < F.ny - 1, zl = k > 0, zr = k < F.nz - 1;
        const T pl = xl ? F.sol[q - 1] : T(0), pr = xr ? F.sol[q + 2] : T(0);
        const V2 pym = yl ? *reinterpret_cast<const V2*>(F.sol + q - sy) : zero2;
        const V2 pyp = yr ? *reinterpret_cast<const V2*>(F.sol + q + sy) : zero2;
        const V2 pzm = zl ? *reinterpret_cast<const V2*>(F.sol + q - sz) : zero2;
        const V2 pzp = zr ? *reinterpret_cast<const V2*>(F.sol + q + sz) : zero2;
        V2 cxp, cym, cyp, czm, czp;
        T cxr;
        if constexpr (kRho) {
          // the children's faces from the density (walls: 0, never used)
          const T* __restrict__ rp = F.rho;
          const V2 r = *reinterpret_cast<const V2*>(rp + q);
          const auto face2 = [&](T kk, bool has, size_t qn) {
            if (!has) return zero2;
            const V2 rn = *reinterpret_cast<const V2*>(rp + qn);
            return V2{rho_face(kk, r.x, rn.x), rho_face(kk, r.y, rn.y)};
          };
          cxp = V2{xl ? rho_face(F.kx, r.x, rp[q - 1]) : T(0), rho_face(F.kx, r.x, r.y)};
          cxr = xr ? rho_face(F.kx, r.y, rp[q + 2]) : T(0);
          cym = face2(F.ky, yl, q - sy);
          cyp = face2(F.ky, yr, q + sy);
          czm = face2(F.kz, zl, q - sz);
          czp = face2(F.kz, zr, q + sz);
        } else {
          cxp = *reinterpret_cast<const V2*>(F.cx + q);
          cxr = xr ? F.cx[q + 2] : T(0);
          cym = *reinterpret_cast<const V2*>(F.cy + q);
          cyp = yr ? *reinterpret_cast<const V2*>(F.cy + q + sy) : zero2;
          czm = *reinterpret_cast<const V2*>(F.cz + q);
          czp = zr ? *reinterpret_cast<const V2*>(F.cz + q + sz) : zero2;
        }
        // child x = i0: neighbours x- (pl, cx[i0]), x+ (p.y, cx[i0+1]); same order as stencil()
        {
          T s = T(0), d = T(0), c;
          if (xl) { c = cxp.x; s += c * pl; d += c; }
          c = cxp.y; s += c * p.y; d += c;
          if (yl) { c = cym.x; s += c * pym.x; d += c; }
          if (yr) { c = cyp.x; s += c * pyp.x; d += c; }
          if (zl) { c = czm.x; s += c * pzm.x; d += c; }
          if (zr) { c = czp.x; s += c * pzp.x; d += c; }
          acc += b.x - (s - d * p.x);
        }
        {
          T s = T(0), d = T(0), c;
          c = cxp.y; s += c * p.x; d += c;
          if (xr) { c = cxr; s += c * pr; d += c; }
          if (yl) { c = cym.y; s += c * pym.y; d += c; }
          if (yr) { c = cyp.y; s += c * pyp.y; d += c; }
          if (zl) { c = czm.y; s += c * pzm.y; d += c; }
          if (zr) { c = czp.y; s += c * pzp.y; d += c; }
          acc += b.y - (s - d * p.y);
        }
      }
  } else {
    for (int dz = 0; dz < F.fz; ++dz)
      for (int dy = 0; dy < F.fy; ++dy)
        for (int dx = 0; dx < F.fx; ++dx) {
          const int i = F.fx * I + dx, j = F.fy * J + dy, k = F.fz * K + dz;
          const size_t q = ((size_t)k * F.ny + j) * F.nx + i;
          T s, d;
          if constexpr (kRho) stencil_rho(F, F.sol, i, j, k, q, s, d);
          else stencil(F, F.sol, i, j, k, q, s, d);
          acc += F.src[q] - (s - d * F.sol[q]);
        }
  }
  const size_t cq = ((size_t)K * C.ny + J) * C.nx + I;
  C.src[cq] = acc * (T(1) / T(F.fx * F.fy * F.fz));
  if (zero_sol) C.sol[cq] = T(0);
}

// Prolongation + correction: fine sol += e_c +/- m/4 per coarsened axis, with
// central slopes m = (e_{c+1} - e_{c-1})/2 and zero-gradient ghosts at walls.
// One thread per coarse cell updates its children; with fx = 2 the two
// x-children are one vector load and store.  Per child the terms are added in
// the order x, y, z, as the oracle does.
template <typename T>
__global__ void __launch_bounds__(256) k_prolong(LevelView<T> F, LevelView<T> C) {
  pdl_enter();
  using V2 = typename Vec2<T>::type;
  const int I = blockIdx.x * blockDim.x + threadIdx.x;
  const int J = blockIdx.y * blockDim.y + threadIdx.y;
  const int K = blockIdx.z;
  if (I >= C.nx || J >= C.ny) return;
  const size_t csy = (size_t)C.nx, csz = (size_t)C.nx * C.ny;
  const size_t cq = (size_t)K * csz + (size_t)J * csy + I;
  const T* e = C.sol;
  const T ec = e[cq];
  T mx = T(0), my = T(0), mz = T(0);
  if (F.fx == 2) mx = T(0.5) * ((I < C.nx - 1 ? e[cq + 1] : ec) - (I > 0 ? e[cq - 1] : ec));
  if (F.fy == 2) my = T(0.5) * ((J < C.ny - 1 ? e[cq + csy] : ec) - (J > 0 ? e[cq - csy] : ec));
  if (F.fz == 2) mz = T(0.5) * ((K < C.nz - 1 ? e[cq + csz] : ec) - (K > 0 ? e[cq - csz] : ec));
  for (int dz = 0; dz < F.fz; ++dz)
    for (int dy = 0; dy < F.fy; ++dy) {
      const int j = F.fy * J + dy, k = F.fz * K + dz;
      T* row = F.sol + ((size_t)k * F.ny + j) * F.nx;
      const T ty = dy ? T(0.25) * my : -(T(0.25) * my);
      const T tz = dz ? T(0.25) * mz : -(T(0.25) * mz);
      if (F.fx == 2) {
        T v0 = ec + -(T(0.25) * mx), v1 = ec + T(0.25) * mx;
        if (F.fy == 2) { v0 += ty; v1 += ty; }
        if (F.fz == 2) { v0 += tz; v1 += tz; }
        V2* pr = reinterpret_cast<V2*>(row) + I;
        V2 cur = *pr;
        cur.x += v0;
        cur.y += v1;
        *pr = cur;
      } else {
        T v = ec;
        if (F.fy == 2) v += ty;
        if (F.fz == 2) v += tz;
        row[I] += v;
      }
    }
}

// FP64 residual r = src - A sol (flux form) with sum r^2.  Blocks stride over (y, z) rows,
// threads over x; r is stored as TO (double, or float for the FP32 cycle).
template <typename TO>
__global__ void __launch_bounds__(kRedThreads) k_residual_norm(LevelView<double> L, TO* r,
                                                               ReduceScratch R, int slot) {
  pdl_enter();
  double acc[1] = {0.0};
  const int rows = L.ny * L.nz;
  for (int row = blockIdx.x; row < rows; row += gridDim.x) {
    const int j = row % L.ny, k = row / L.ny;
    for (int i = threadIdx.x; i < L.nx; i += blockDim.x) {
      const size_t q = ((size_t)k * L.ny + j) * L.nx + i;
      const double rr = L.src[q] - flux_sum(L, L.sol, i, j, k, q);
      if (r) r[q] = (TO)rr;
      acc[0] += rr * rr;
    }
  }
  grid_sum_finish<1>(acc, R, slot);
}

// q = A d and sum d.q (the flexible-CG matrix product), rows as k_residual_norm.
__global__ void __launch_bounds__(kRedThreads) k_apply_dot(LevelView<double> L,
                                                           const double* __restrict__ dvec,
                                                           double* qvec, ReduceScratch R,
                                                           int slot) {
  double acc[1] = {0.0};
  const int rows = L.ny * L.nz;
  for (int row = blockIdx.x; row < rows; row += gridDim.x) {
    const int j = row % L.ny, k = row / L.ny;
    for (int i = threadIdx.x; i < L.nx; i += blockDim.x) {
      const size_t q = ((size_t)k * L.ny + j) * L.nx + i;
      double s, d;
      stencil(L, dvec, i, j, k, q, s, d);
      const double a = s - d * dvec[q];
      qvec[q] = a;
      acc[0] += dvec[q] * a;
    }
  }
  grid_sum_finish<1>(acc, R, slot);
}

// Dense solve of the coarsest level, one block: x = Minv b; one refinement
// step when max|b - A x| > 1e-10 (mg_find_error / mg_solve_correct,
// "DomainDecomposition/3D/lib/data/tree_multigrid.f90:175-238"); mean projection
// (multigrid_final_exact's compatibility_sol, multigrid_solver.f90:100).
template <typename T>
__global__ void __launch_bounds__(kMaxCoarse) k_coarse_solve(int n, const T* __restrict__ minv,
                                                             const T* __restrict__ a,
                                                             const T* __restrict__ b, T* x) {
  pdl_enter();
  __shared__ T sb[kMaxCoarse], sx[kMaxCoarse], se[kMaxCoarse];
  __shared__ T red[kMaxCoarse];
  __shared__ int refine;
  const int t = threadIdx.x;
  if (t == 0) refine = 0;
  if (t < n) sb[t] = b[t];
  __syncthreads();
  if (t < n) {
    T acc = T(0);
    for (int q = 0; q < n; ++q) acc += minv[t * n + q] * sb[q];
    sx[t] = acc;
  }
  __syncthreads();
  if (t < n) {
    T e = sb[t];
    for (int q = 0; q < n; ++q) e -= a[t * n + q] * sx[q];
    se[t] = e;
    if (fabs((double)e) > 1e-10) atomicOr(&refine, 1);
  }
  __syncthreads();
  if (refine && t < n) {
    T acc = T(0);
    for (int q = 0; q < n; ++q) acc += minv[t * n + q] * se[q];
    sx[t] += acc;
  }
  __syncthreads();
  // mean projection, summed in index order by thread 0 (n <= 64)
  if (t == 0) {
    T s = T(0);
    for (int q = 0; q < n; ++q) s += sx[q];
    red[0] = s / T(n);
  }
  __syncthreads();
  if (t < n) x[t] = sx[t] - red[0];
}

// Coarsest-level operator and its inverse, one block, FP64.  The dense
// Neumann matrix A is singular (constant null space) and negative
// semi-definite; M = s 11^T/n - A (s = mean diagonal) is symmetric positive
// definite, and -M^{-1} b is the mean-free solution of A x = b for a
// mean-free b.  M = L L^T by Cholesky in shared memory, W = L^{-1} column by
// column, M^{-1} = W^T W: about n^3/2 multiply-adds instead of Gauss-Jordan's
// 2n^3.  The reference LU-factors the singular matrix with LAPACK dgesv
// instead ("DomainDecomposition/3D/lib/data/tree_multigrid.f90:134-173").
__global__ void __launch_bounds__(256) k_coarse_invert(LevelView<double> C, double* minv,
                                                       double* adense, float* minv32,
                                                       float* adense32) {
  extern __shared__ double smem[];
  const int n = C.nx * C.ny * C.nz;
  double* M = smem;                   // n x n, becomes L (lower triangle)
  double* W = smem + (size_t)n * n;   // n x n, becomes L^{-1} (lower triangle)
  __shared__ double dsum_sh;
  const int t = threadIdx.x, nt = blockDim.x;
  for (int e = t; e < n * n; e += nt) adense[e] = 0.0;
  __syncthreads();
  if (t == 0) {
    // assemble A in the oracle's order (serial, n <= 64)
    double dsum = 0.0;
    for (int k = 0; k < C.nz; ++k)
      for (int j = 0; j < C.ny; ++j)
        for (int i = 0; i < C.nx; ++i) {
          const int q = (k * C.ny + j) * C.nx + i;
          double d = 0.0, c;
          if (i > 0) { c = C.cx[q]; adense[q * n + q - 1] += c; d += c; }
          if (i < C.nx - 1) { c = C.cx[q + 1]; adense[q * n + q + 1] += c; d += c; }
          if (j > 0) { c = C.cy[q]; adense[q * n + q - C.nx] += c; d += c; }
          if (j < C.ny - 1) { c = C.cy[q + C.nx]; adense[q * n + q + C.nx] += c; d += c; }
          if (k > 0) { c = C.cz[q]; adense[q * n + q - C.nx * C.ny] += c; d += c; }
          if (k < C.nz - 1) { c = C.cz[q + C.nx * C.ny]; adense[q * n + q + C.nx * C.ny] += c; d += c; }
          adense[q * n + q] -= d;
          dsum += d;
        }
    double s = n > 0 ? dsum / n : 1.0;
    if (s <= 0.0) s = 1.0;
    dsum_sh = s;
  }
  __syncthreads();
  const double sn = dsum_sh / n;
  for (int e = t; e < n * n; e += nt) {
    M[e] = sn - adense[e];
    W[e] = 0.0;
  }
  __syncthreads();
  // right-looking Cholesky, lower triangle in place
  for (int j = 0; j < n; ++j) {
    if (t == 0) M[j * n + j] = sqrt(M[j * n + j]);
    __syncthreads();
    const double djj = M[j * n + j];
    for (int i = j + 1 + t; i < n; i += nt) M[i * n + j] /= djj;
    __syncthreads();
    const int m = n - j - 1;  // trailing block (j+1..n-1)^2, lower part
    for (int e = t; e < m * m; e += nt) {
      const int i = j + 1 + e / m, k = j + 1 + e % m;
      if (k <= i) M[i * n + k] -= M[i * n + j] * M[k * n + j];
    }
    __syncthreads();
  }
  // W = L^{-1}: forward substitution, one column per thread
  for (int c = t; c < n; c += nt) {
    W[c * n + c] = 1.0 / M[c * n + c];
    for (int i = c + 1; i < n; ++i) {
      double acc = 0.0;
      for (int k = c; k < i; ++k) acc += M[i * n + k] * W[k * n + c];
      W[i * n + c] = -acc / M[i * n + i];
    }
  }
  __syncthreads();
  // (A - s 11^T/n)^{-1} = -M^{-1} = -W^T W
  for (int e = t; e < n * n; e += nt) {
    const int r = e / n, q = e % n;
    double acc = 0.0;
    for (int k = max(r, q); k < n; ++k) acc += W[k * n + r] * W[k * n + q];
    minv[e] = -acc;
    if (minv32) minv32[e] = (float)(-acc);
    if (adense32) adense32[e] = (float)adense[e];
  }
}

// Coarse face coefficients, rediscretised on spacing 2h from the mean of the
// fine face coefficients covering each coarse face: coe_c = mean(coe_f)/f^2
// along a coarsened axis (beta_c = mean beta_f).  The reference multigrid is
// constant-coefficient and has no counterpart.
__global__ void __launch_bounds__(256) k_coarsen(LevelView<double> F, double* cx, double* cy,
                                                 double* cz, int cnx, int cny, int cnz) {
  const int I = blockIdx.x * blockDim.x + threadIdx.x;
  const int J = blockIdx.y * blockDim.y + threadIdx.y;
  const int K = blockIdx.z;
  if (I >= cnx || J >= cny) return;
  const size_t cq = ((size_t)K * cny + J) * cnx + I;
  const double tang = 1.0 / (double)(F.fx * F.fy * F.fz);
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const double* fc = a == 0 ? F.cx : (a == 1 ? F.cy : F.cz);
    double* cc = a == 0 ? cx : (a == 1 ? cy : cz);
    const int idx = a == 0 ? I : (a == 1 ? J : K);
    const int fa = a == 0 ? F.fx : (a == 1 ? F.fy : F.fz);
    if (idx == 0 || fa == 1) { cc[cq] = 0.0; continue; }
    double acc = 0.0;
    for (int dz = 0; dz < F.fz; ++dz)
      for (int dy = 0; dy < F.fy; ++dy)
        for (int dx = 0; dx < F.fx; ++dx) {
          if ((a == 0 && dx) || (a == 1 && dy) || (a == 2 && dz)) continue;
          const size_t fq = ((size_t)(F.fz * K + dz) * F.ny + (F.fy * J + dy)) * F.nx + (F.fx * I + dx);
          acc += fc[fq];
        }
    acc *= tang * fa;
    cc[cq] = acc / (double)(fa * fa);
  }
}

__global__ void __launch_bounds__(256) k_idiag(LevelView<double> L, double* idiag) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i >= L.nx || j >= L.ny) return;
  const size_t sy = (size_t)L.nx, sz = (size_t)L.nx * L.ny;
  const size_t q = (size_t)k * sz + (size_t)j * sy + i;
  double d = 0.0;
  if (i > 0) d += L.cx[q];
  if (i < L.nx - 1) d += L.cx[q + 1];
  if (j > 0) d += L.cy[q];
  if (j < L.ny - 1) d += L.cy[q + sy];
  if (k > 0) d += L.cz[q];
  if (k < L.nz - 1) d += L.cz[q + sz];
  idiag[q] = d > 0.0 ? 1.0 / d : 0.0;
}

__global__ void k_to_float(const double* __restrict__ a, float* __restrict__ b, size_t n) {
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n;
       q += (size_t)gridDim.x * blockDim.x)
    b[q] = (float)a[q];
}

}  // namespace

// ---------------------------------------------------------------------------
template <typename T>
void launch_smooth(cudaStream_t s, const LevelView<T>& L, int color, bool zero_guess) {
  const dim3 blk(32, 8, 1);
  const dim3 grd(cdiv((size_t)(L.nx + 1) / 2, 32), cdiv((size_t)L.ny, 8), (unsigned)L.nz);
  if constexpr (std::is_same<T, float>::value) {
    if (L.split) {
      launch_smooth_split(s, L, color, zero_guess);
      return;
    }
    if (L.rho) {
      if (zero_guess) launch_pdl(k_smooth<T, false, true, true>, grd, blk, 0, s, L, color);
      else launch_pdl(k_smooth<T, false, false, true>, grd, blk, 0, s, L, color);
      return;
    }
  }
  if (L.idiag) {
    if (zero_guess) launch_pdl(k_smooth<T, true, true, false>, grd, blk, 0, s, L, color);
    else launch_pdl(k_smooth<T, true, false, false>, grd, blk, 0, s, L, color);
  } else {
    if (zero_guess) launch_pdl(k_smooth<T, false, true, false>, grd, blk, 0, s, L, color);
    else launch_pdl(k_smooth<T, false, false, false>, grd, blk, 0, s, L, color);
  }
}

template <typename T>
void launch_restrict(cudaStream_t s, const LevelView<T>& F, const LevelView<T>& C, bool zero_sol) {
  const dim3 blk(32, 8, 1);
  const dim3 grd(cdiv((size_t)C.nx, 32), cdiv((size_t)C.ny, 8), (unsigned)C.nz);
  if constexpr (std::is_same<T, float>::value) {
    if (F.split) {
      launch_restrict_split(s, F, C, zero_sol);
      return;
    }
    if (F.rho) {
      launch_pdl(k_restrict<T, true>, grd, blk, 0, s, F, C, zero_sol ? 1 : 0);
      return;
    }
  }
  launch_pdl(k_restrict<T, false>, grd, blk, 0, s, F, C, zero_sol ? 1 : 0);
}

template <typename T>
void launch_prolong(cudaStream_t s, const LevelView<T>& F, const LevelView<T>& C) {
  const dim3 blk(32, 8, 1);
  const dim3 grd(cdiv((size_t)C.nx, 32), cdiv((size_t)C.ny, 8), (unsigned)C.nz);
  if constexpr (std::is_same<T, float>::value) {
    if (F.split) {
      launch_prolong_split(s, F, C);
      return;
    }
  }
  launch_pdl(k_prolong<T>, grd, blk, 0, s, F, C);
}

// Blocks for a grid-stride reduction: 8 per SM, at most one per row.  The SM
// count is read once per process (every GPU of the target has the same).
int reduce_blocks_for(size_t rows) {
  static int sms = 0;
  if (sms == 0) {
    int dev = 0, v = 152;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) v = 152;
    sms = v;
  }
  const size_t cap = (size_t)sms * 8;
  return (int)(rows < cap ? (rows > 0 ? rows : 1) : cap);
}

template <typename TO>
void launch_residual_norm(cudaStream_t s, const LevelView<double>& L, TO* r,
                          const ReduceScratch& R, int slot) {
  const int blocks = std::min(reduce_blocks_for((size_t)L.ny * L.nz), R.max_blocks);
  launch_pdl(k_residual_norm<TO>, dim3(blocks), dim3(kRedThreads), 0, s, L, r, R, slot);
}

void launch_apply_dot(cudaStream_t s, const LevelView<double>& L, const double* d, double* q,
                      const ReduceScratch& R, int slot) {
  const int blocks = std::min(reduce_blocks_for((size_t)L.ny * L.nz), R.max_blocks);
  k_apply_dot<<<blocks, kRedThreads, 0, s>>>(L, d, q, R, slot);
}

template <typename T>
void launch_coarse_solve(cudaStream_t s, int n, const T* minv, const T* adense, const T* b, T* x) {
  launch_pdl(k_coarse_solve<T>, dim3(1), dim3(kMaxCoarse), 0, s, n, minv, adense, b, x);
}

void launch_coarse_invert(cudaStream_t s, const LevelView<double>& C, double* minv,
                          double* adense, float* minv32, float* adense32) {
  const int n = C.nx * C.ny * C.nz;
  const size_t shm = (size_t)2 * n * n * sizeof(double);
  cudaFuncSetAttribute(k_coarse_invert, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm);
  k_coarse_invert<<<1, 256, shm, s>>>(C, minv, adense, minv32, adense32);
}

void launch_coarsen(cudaStream_t s, const LevelView<double>& F, double* cx, double* cy,
                    double* cz, int cnx, int cny, int cnz) {
  const dim3 blk(32, 8, 1);
  const dim3 grd(cdiv((size_t)cnx, 32), cdiv((size_t)cny, 8), (unsigned)cnz);
  k_coarsen<<<grd, blk, 0, s>>>(F, cx, cy, cz, cnx, cny, cnz);
}

void launch_idiag(cudaStream_t s, const LevelView<double>& L, double* idiag) {
  const dim3 blk(32, 8, 1);
  const dim3 grd(cdiv((size_t)L.nx, 32), cdiv((size_t)L.ny, 8), (unsigned)L.nz);
  k_idiag<<<grd, blk, 0, s>>>(L, idiag);
}

void launch_to_float(cudaStream_t s, const double* a, float* b, size_t n) {
  const unsigned blocks = (unsigned)std::min<size_t>(cdiv(n, 256), 152 * 16);
  k_to_float<<<blocks > 0 ? blocks : 1, 256, 0, s>>>(a, b, n);
}

template void launch_smooth<double>(cudaStream_t, const LevelView<double>&, int, bool);
template void launch_smooth<float>(cudaStream_t, const LevelView<float>&, int, bool);
template void launch_restrict<double>(cudaStream_t, const LevelView<double>&,
                                      const LevelView<double>&, bool);
template void launch_restrict<float>(cudaStream_t, const LevelView<float>&,
                                     const LevelView<float>&, bool);
template void launch_prolong<double>(cudaStream_t, const LevelView<double>&,
                                     const LevelView<double>&);
template void launch_prolong<float>(cudaStream_t, const LevelView<float>&,
                                    const LevelView<float>&);
template void launch_residual_norm<double>(cudaStream_t, const LevelView<double>&, double*,
                                           const ReduceScratch&, int);
template void launch_residual_norm<float>(cudaStream_t, const LevelView<double>&, float*,
                                          const ReduceScratch&, int);
template void launch_coarse_solve<double>(cudaStream_t, int, const double*, const double*,
                                          const double*, double*);
template void launch_coarse_solve<float>(cudaStream_t, int, const float*, const float*,
                                         const float*, float*);

}  // namespace gbmg
