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
#include "mg_cells.cuh"
#include "pdl.cuh"
#include "reduce.cuh"

namespace gbmg {

namespace {

inline unsigned cdiv(size_t a, unsigned b) { return (unsigned)((a + b - 1) / b); }

using namespace cells;

// One colour of a red-black sweep, one thread per cell of the colour.
template <typename T, bool kIdiag, bool kZero, bool kRho>
__global__ void __launch_bounds__(256) k_smooth(LevelView<T> L, int color) {
  pdl_enter();
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (j >= L.ny) return;
  const int i = 2 * (blockIdx.x * blockDim.x + threadIdx.x) + ((j + k + color) & 1);
  if (i >= L.nx) return;
  smooth_cell<T, kIdiag, kZero, kRho>(L, i, j, k);
}

// Fused residual + restriction, one thread per coarse cell.
template <typename T, bool kRho>
__global__ void __launch_bounds__(256) k_restrict(LevelView<T> F, LevelView<T> C, int zero_sol) {
  pdl_enter();
  const int I = blockIdx.x * blockDim.x + threadIdx.x;
  const int J = blockIdx.y * blockDim.y + threadIdx.y;
  const int K = blockIdx.z;
  if (I >= C.nx || J >= C.ny) return;
  restrict_cell<T, kRho>(F, C, I, J, K, zero_sol);
}

// Prolongation + correction, one thread per coarse cell.
template <typename T>
__global__ void __launch_bounds__(256) k_prolong(LevelView<T> F, LevelView<T> C) {
  pdl_enter();
  const int I = blockIdx.x * blockDim.x + threadIdx.x;
  const int J = blockIdx.y * blockDim.y + threadIdx.y;
  const int K = blockIdx.z;
  if (I >= C.nx || J >= C.ny) return;
  prolong_cell<T>(F, C, I, J, K);
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

// Coarsest-level operator and its inverse, FP64.  The dense Neumann matrix A
// is singular (constant null space) and negative semi-definite;
// M = s 11^T/n - A (s = mean diagonal) is symmetric positive definite, and
// -M^{-1} b is the mean-free solution of A x = b for a mean-free b.
// M = L L^T by Cholesky in shared memory (one block), W = L^{-1} one column
// per block, M^{-1} = W^T W one row per block: about n^3/2 multiply-adds
// instead of Gauss-Jordan's 2n^3, and the two triangular products, which are
// FP64-pipe bound on one SM, spread over n SMs.  The reference LU-factors the
// singular matrix with LAPACK dgesv instead
// ("DomainDecomposition/3D/lib/data/tree_multigrid.f90:134-173").
//
// work holds L (n x n, lower triangle), 1/L_jj (n) and W (n x n).
__global__ void __launch_bounds__(256) k_coarse_factor(LevelView<double> C, double* adense,
                                                       float* adense32, double* work) {
  extern __shared__ double smem[];
  const int n = C.nx * C.ny * C.nz;
  double* M = smem;  // n x n, becomes L (lower triangle)
  __shared__ double dsum_sh;
  __shared__ double drow[kMaxCoarse];
  const int t = threadIdx.x, nt = blockDim.x;
  for (int e = t; e < n * n; e += nt) M[e] = 0.0;
  __syncthreads();
  // assemble A, one row per thread; the diagonal sums its faces in the order
  // x-, x+, y-, y+, z-, z+ and the mean diagonal sums the rows in order
  if (t < n) {
    const int q = t, sy = C.nx, sz = C.nx * C.ny;
    const int i = q % C.nx, j = (q / C.nx) % C.ny, k = q / sz;
    const double cxl = i > 0 ? C.cx[q] : 0.0, cxr = i < C.nx - 1 ? C.cx[q + 1] : 0.0;
    const double cyl = j > 0 ? C.cy[q] : 0.0, cyr = j < C.ny - 1 ? C.cy[q + sy] : 0.0;
    const double czl = k > 0 ? C.cz[q] : 0.0, czr = k < C.nz - 1 ? C.cz[q + sz] : 0.0;
    double d = 0.0;
    if (i > 0) { M[q * n + q - 1] = cxl; d += cxl; }
    if (i < C.nx - 1) { M[q * n + q + 1] = cxr; d += cxr; }
    if (j > 0) { M[q * n + q - sy] = cyl; d += cyl; }
    if (j < C.ny - 1) { M[q * n + q + sy] = cyr; d += cyr; }
    if (k > 0) { M[q * n + q - sz] = czl; d += czl; }
    if (k < C.nz - 1) { M[q * n + q + sz] = czr; d += czr; }
    M[q * n + q] = -d;
    drow[q] = d;
  }
  __syncthreads();
  if (t == 0) {
    double dsum = 0.0;
    for (int q = 0; q < n; ++q) dsum += drow[q];
    double s = n > 0 ? dsum / n : 1.0;
    if (s <= 0.0) s = 1.0;
    dsum_sh = s;
  }
  __syncthreads();
  const double sn = dsum_sh / n;
  for (int e = t; e < n * n; e += nt) {
    const double a = M[e];
    adense[e] = a;
    if (adense32) adense32[e] = (float)a;
    M[e] = sn - a;
  }
  __syncthreads();
  // right-looking Cholesky, lower triangle in place; the trailing update is
  // walked as a 16 x 16 thread grid over (row, column) without divisions
  double* rdiag = work + (size_t)n * n;  // 1/L_jj
  __shared__ double rd_sh;
  const int tx = t % 16, ty = t / 16;
  for (int j = 0; j < n; ++j) {
    if (t == 0) {
      const double d = sqrt(M[j * n + j]);
      M[j * n + j] = d;
      rd_sh = 1.0 / d;
      rdiag[j] = rd_sh;
    }
    __syncthreads();
    const double rjj = rd_sh;
    for (int i = j + 1 + t; i < n; i += nt) M[i * n + j] *= rjj;
    __syncthreads();
    for (int i = j + 1 + ty; i < n; i += 16) {
      const double lij = M[i * n + j];
      for (int k = j + 1 + tx; k <= i; k += 16) M[i * n + k] -= lij * M[k * n + j];
    }
    __syncthreads();
  }
  for (int e = t; e < n * n; e += nt) work[e] = M[e];
}

// W = L^{-1}, column c in block c (one warp): row by row forward
// substitution, the dot product of each row split over the lanes.
__global__ void __launch_bounds__(32) k_coarse_lower_inv(int n, double* work) {
  const double* Lm = work;
  const double* rdiag = work + (size_t)n * n;
  double* W = work + (size_t)n * n + n;
  __shared__ double col[kMaxCoarse];
  const int c = blockIdx.x, lane = threadIdx.x;
  for (int i = lane; i < n; i += 32) col[i] = 0.0;
  __syncwarp();
  if (lane == 0) col[c] = rdiag[c];
  __syncwarp();
  for (int i = c + 1; i < n; ++i) {
    double acc = 0.0;
    for (int k = c + lane; k < i; k += 32) acc += Lm[(size_t)i * n + k] * col[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) col[i] = -acc * rdiag[i];
    __syncwarp();
  }
  for (int i = lane; i < n; i += 32) W[(size_t)i * n + c] = col[i];
}

// (A - s 11^T/n)^{-1} = -M^{-1} = -W^T W, row r in block r.
__global__ void __launch_bounds__(kMaxCoarse) k_coarse_gram(int n, const double* __restrict__ work,
                                                           double* minv, float* minv32) {
  const double* W = work + (size_t)n * n + n;
  const int r = blockIdx.x, q = threadIdx.x;
  if (q >= n) return;
  double acc = 0.0;
  for (int k = max(r, q); k < n; ++k) acc += W[(size_t)k * n + r] * W[(size_t)k * n + q];
  minv[(size_t)r * n + q] = -acc;
  if (minv32) minv32[(size_t)r * n + q] = (float)(-acc);
}

// Coarse face coefficients, rediscretised on spacing 2h from the mean of the
// fine face coefficients covering each coarse face: coe_c = mean(coe_f)/f^2
// along a coarsened axis (beta_c = mean beta_f).  The reference multigrid is
// constant-coefficient and has no counterpart.
// With c32: the coefficients rounded to float into c32[0..2] as well.
__global__ void __launch_bounds__(256) k_coarsen(LevelView<double> F, double* cx, double* cy,
                                                 double* cz, int cnx, int cny, int cnz,
                                                 Float3Out c32) {
  const int I = blockIdx.x * blockDim.x + threadIdx.x;
  const int J = blockIdx.y * blockDim.y + threadIdx.y;
  const int K = blockIdx.z;
  if (I >= cnx || J >= cny) return;
  const size_t cq = ((size_t)K * cny + J) * cnx + I;
  const size_t sy = (size_t)F.nx, sz = (size_t)F.nx * F.ny;
  const size_t q0 = (size_t)F.fz * K * sz + (size_t)F.fy * J * sy + (size_t)F.fx * I;
  if (F.fx <= 2 && F.fy <= 2 && F.fz <= 2) {
    // all (at most 12) loads issued before the sums, which keep the order
    // dz, dy, dx of the general loop below.  The factors are powers of two, so
    // 1/(fx fy fz) and the division by fa^2 are exact products: GB300 runs an
    // FP64 division as a long sequence on its slow FP64 pipe.
    const int f3 = F.fx * F.fy * F.fz;
    const double tang = f3 == 1 ? 1.0 : (f3 == 2 ? 0.5 : (f3 == 4 ? 0.25 : 0.125));
    double t[3][4];
    bool use[3][4];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const double* fc = a == 0 ? F.cx : (a == 1 ? F.cy : F.cz);
      const int idx = a == 0 ? I : (a == 1 ? J : K);
      const int fa = a == 0 ? F.fx : (a == 1 ? F.fy : F.fz);
      const bool live = idx > 0 && fa > 1;
#pragma unroll
      for (int m = 0; m < 4; ++m) {
        // the two tangential offsets of slot m, in the loop order z, y, x
        const int hi = m >> 1, lo = m & 1;
        const int dz = a == 2 ? 0 : hi, dy = a == 1 ? 0 : (a == 0 ? lo : hi), dx = a == 0 ? 0 : lo;
        use[a][m] = live && dz < F.fz && dy < F.fy && dx < F.fx;
        t[a][m] = use[a][m] ? fc[q0 + dz * sz + dy * sy + dx] : 0.0;
      }
    }
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      double* cc = a == 0 ? cx : (a == 1 ? cy : cz);
      const int idx = a == 0 ? I : (a == 1 ? J : K);
      const int fa = a == 0 ? F.fx : (a == 1 ? F.fy : F.fz);
      double v = 0.0;
      if (!(idx == 0 || fa == 1)) {
        double acc = 0.0;
#pragma unroll
        for (int m = 0; m < 4; ++m)
          if (use[a][m]) acc += t[a][m];
        acc *= tang * fa;
        v = acc * (fa == 2 ? 0.25 : 1.0);
      }
      cc[cq] = v;
      if (c32.p[a]) c32.p[a][cq] = (float)v;
    }
    return;
  }
  const double tang = 1.0 / (double)(F.fx * F.fy * F.fz);
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const double* fc = a == 0 ? F.cx : (a == 1 ? F.cy : F.cz);
    double* cc = a == 0 ? cx : (a == 1 ? cy : cz);
    const int idx = a == 0 ? I : (a == 1 ? J : K);
    const int fa = a == 0 ? F.fx : (a == 1 ? F.fy : F.fz);
    double v = 0.0;
    if (!(idx == 0 || fa == 1)) {
      double acc = 0.0;
      for (int dz = 0; dz < F.fz; ++dz)
        for (int dy = 0; dy < F.fy; ++dy)
          for (int dx = 0; dx < F.fx; ++dx) {
            if ((a == 0 && dx) || (a == 1 && dy) || (a == 2 && dz)) continue;
            acc += fc[q0 + dz * sz + dy * sy + dx];
          }
      acc *= tang * fa;
      v = acc / (double)(fa * fa);
    }
    cc[cq] = v;
    if (c32.p[a]) c32.p[a][cq] = (float)v;
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
  stride4(n, [&](size_t q) { return a[q]; }, [&](size_t q, double v) { b[q] = (float)v; });
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
void launch_prolong(cudaStream_t s, const LevelView<T>& F, const LevelView<T>& C, int live) {
  const dim3 blk(32, 8, 1);
  const dim3 grd(cdiv((size_t)C.nx, 32), cdiv((size_t)C.ny, 8), (unsigned)C.nz);
  if constexpr (std::is_same<T, float>::value) {
    if (F.split) {
      launch_prolong_split(s, F, C, live);
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
                          double* adense, float* minv32, float* adense32, double* work) {
  const int n = C.nx * C.ny * C.nz;
  const size_t shm = (size_t)n * n * sizeof(double);
  cudaFuncSetAttribute(k_coarse_factor, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm);
  k_coarse_factor<<<1, 256, shm, s>>>(C, adense, adense32, work);
  k_coarse_lower_inv<<<n, 32, 0, s>>>(n, work);
  k_coarse_gram<<<n, kMaxCoarse, 0, s>>>(n, work, minv, minv32);
}

void launch_coarsen(cudaStream_t s, const LevelView<double>& F, double* cx, double* cy,
                    double* cz, int cnx, int cny, int cnz, Float3Out c32) {
  const dim3 blk(32, 8, 1);
  const dim3 grd(cdiv((size_t)cnx, 32), cdiv((size_t)cny, 8), (unsigned)cnz);
  k_coarsen<<<grd, blk, 0, s>>>(F, cx, cy, cz, cnx, cny, cnz, c32);
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
                                     const LevelView<double>&, int);
template void launch_prolong<float>(cudaStream_t, const LevelView<float>&,
                                    const LevelView<float>&, int);
template void launch_residual_norm<double>(cudaStream_t, const LevelView<double>&, double*,
                                           const ReduceScratch&, int);
template void launch_residual_norm<float>(cudaStream_t, const LevelView<double>&, float*,
                                          const ReduceScratch&, int);
template void launch_coarse_solve<double>(cudaStream_t, int, const double*, const double*,
                                          const double*, double*);
template void launch_coarse_solve<float>(cudaStream_t, int, const float*, const float*,
                                         const float*, float*);

}  // namespace gbmg
