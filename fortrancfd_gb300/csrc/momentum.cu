// Adams-Bashforth momentum step of the two-phase solvers on sm_103a:
// ns_ab_solver_SOR's explicit part ("Two phase flows/newOpenMP/2D/src/
// ns_solver/admas_bashforth_solver.f90", 3D "…/3D+IBM/src/ns_solver/
// admas_bashforth_solver.f90") around the pressure projection.
//
//   k_ns_diffusion  velsrc%tmp = sec_part1 + sec_part2 + sec_part3
//                   (ns_ab_diff.f90): viscous term, interface-viscosity term,
//                   gravity and surface tension, from the old fields; once per
//                   step (it does not depend on the advecting velocity).
//   k_ns_advance    find_stag_vel's averages of vel%tmp, the second-order
//                   upwind advection of vel%old (ns_ab_adv_source_sec),
//                   velsrc%now = advection + velsrc%tmp (ns_ab_setup) and the
//                   AB2 predictor (ns_ab_predictor), fused: one pass per
//                   predictor-projection iteration.
//   k_velbc         velbc (bcs.f90) on the ghost shell: each ghost value is
//                   the composition of the reference's x, y and z passes,
//                   computed directly from the interior value it mirrors.
//   k_ns_change     ns_check_convergence_vel: max and sum of squares of
//                   vel%now - vel%tmp.
//
// Layout: every array is the reference's ghost-padded box with g >= 2 ghost
// layers and the strides sy, sz of the caller (x contiguous).  Kernels take
// the address of the reference's element (1,1,1) of each array, so element
// (i,j,k) of the 1-based reference indices sits at (i-1) + (j-1) sy + (k-1) sz
// for cell arrays and face arrays alike (u(i,j,k) is the face i+1/2).
//
// Arithmetic: FP64, every expression in the reference's operand order, and
// this translation unit is compiled with -fmad=false, so no multiply-add is
// contracted: each value is the same double rounding as the reference's (and
// the oracle's, built with -ffp-contract=off), bit for bit.  The reference
// divides a lot (by dx, dx^2, Re, rho Re, ...), and GB300's FP64 pipe is
// narrow: quotients by a divisor used more than once come from its correctly
// rounded reciprocal without a division (fdiv.cuh), which yields the same
// doubles; the rest are IEEE divisions.
#include <algorithm>

#include "fdiv.cuh"
#include "gbmg_internal.h"
#include "reduce.cuh"

namespace gbmg {

namespace {

constexpr int kNsBx = 32, kNsBy = 8;

// a / b for a constant divisor b with reciprocal y = RN(1/b)
__device__ __forceinline__ double cdiv(const NsArgs& a, double x, double b, double y) {
  return a.fast ? div_known(x, b, y) : x / b;
}

// signed: ghost elements lie before element (1,1,1)
__device__ __forceinline__ int64_t ns_at(const NsArgs& a, int i, int j, int k) {
  return (int64_t)(i - 1) + (int64_t)(j - 1) * a.sy + (int64_t)(k - 1) * a.sz;
}

template <bool kThree>
__global__ void __launch_bounds__(kNsBx * kNsBy)
    k_ns_diffusion(NsArgs a, const double* __restrict__ U, const double* __restrict__ V,
                   const double* __restrict__ W, const double* __restrict__ R,
                   const double* __restrict__ M, const double* __restrict__ D,
                   const double* __restrict__ P, const double* __restrict__ N1,
                   const double* __restrict__ N2, const double* __restrict__ N3,
                   const double* __restrict__ CV, double* __restrict__ TU,
                   double* __restrict__ TV, double* __restrict__ TW) {
  const int i = blockIdx.x * kNsBx + threadIdx.x + 1;
  const int j = blockIdx.y * kNsBy + threadIdx.y + 1;
  const int k = blockIdx.z + 1;
  if (i > a.nx || j > a.ny) return;
  const int64_t sx = 1, sy = a.sy, sz = a.sz;
  const int64_t q = ns_at(a, i, j, k);
  const double dx = a.dx, dy = a.dy, dz = a.dz;
  const double dx2 = dx * dx, dy2 = dy * dy, dz2 = dz * dz;
  const double re = a.re, c1 = 1.0 - a.mu_12;
  const bool sf = a.btn_sf != 0.0;
  double rho, mu, mr, rr, yr, delta, curv, xx, yy, zz, t;
  double ux, uy, uz, vx, vy, vz, wx, wy, wz, phix, phiy, phiz, dxx, dyy, dzz;
  // x / (rho re): three quotients share the divisor, so one IEEE division
  // gives its reciprocal and the quotients follow without dividing
#define NS_DRR(x) (a.fast ? div_known_checked((x), rr, yr) : (x) / rr)
  // ---- x: u at (i+1/2, j, k) ----
  rho = 0.5 * (R[q] + R[q + sx]);
  mu = 0.5 * (M[q] + M[q + sx]);
  mr = mu / rho;
  xx = cdiv(a, (U[q + sx] - 2.0 * U[q]) + U[q - sx], dx2, a.rdx2);
  yy = cdiv(a, (U[q + sy] - 2.0 * U[q]) + U[q - sy], dy2, a.rdy2);
  t = cdiv(a, mr * xx, re, a.rre) + cdiv(a, mr * yy, re, a.rre);
  if (kThree) {
    zz = cdiv(a, (U[q + sz] - 2.0 * U[q]) + U[q - sz], dz2, a.rdz2);
    t = t + cdiv(a, mr * zz, re, a.rre);
  }
  delta = 0.5 * (D[q] + D[q + sx]);
  rr = rho * re;
  yr = a.fast ? 1.0 / rr : 0.0;
  ux = cdiv(a, 0.5 * (U[q + sx] - U[q - sx]), dx, a.rdx);
  uy = cdiv(a, 0.5 * (U[q + sy] - U[q - sy]), dy, a.rdy);
  vx = cdiv(a, 0.5 * (((V[q + sx] - V[q]) + V[q + sx - sy]) - V[q - sy]), dx, a.rdx);
  phix = cdiv(a, P[q + sx] - P[q], dx, a.rdx);
  phiy = cdiv(a, 0.25 * (((P[q + sx + sy] - P[q + sx - sy]) + P[q + sy]) - P[q - sy]), dy, a.rdy);
  dxx = NS_DRR(c1 * delta * phix * 2.0 * ux);
  dyy = NS_DRR(c1 * delta * phiy * (uy + vx));
  t = (t + dxx) + dyy;
  if (kThree) {
    uz = cdiv(a, 0.5 * (U[q + sz] - U[q - sz]), dz, a.rdz);
    wx = cdiv(a, 0.5 * (((W[q + sx] - W[q]) + W[q + sx - sz]) - W[q - sz]), dx, a.rdx);
    phiz = cdiv(a, 0.25 * (((P[q + sx + sz] - P[q + sx - sz]) + P[q + sz]) - P[q - sz]), dz, a.rdz);
    dzz = NS_DRR(c1 * delta * phiz * (uz + wx));
    t = t + dzz;
  }
  t = t + a.gterm[0];
  if (sf) {
    curv = (CV[q] + CV[q + sx]) / 2.0;
    phix = 0.5 * (N1[q] + N1[q + sx]);
    t = t - a.btn_sf * curv * delta * phix / (a.we * rho);
  }
  TU[q] = t;
  // ---- y: v at (i, j+1/2, k) ----
  rho = 0.5 * (R[q] + R[q + sy]);
  mu = 0.5 * (M[q] + M[q + sy]);
  mr = mu / rho;
  xx = cdiv(a, (V[q + sx] - 2.0 * V[q]) + V[q - sx], dx2, a.rdx2);
  yy = cdiv(a, (V[q + sy] - 2.0 * V[q]) + V[q - sy], dy2, a.rdy2);
  t = cdiv(a, mr * xx, re, a.rre) + cdiv(a, mr * yy, re, a.rre);
  if (kThree) {
    zz = cdiv(a, (V[q + sz] - 2.0 * V[q]) + V[q - sz], dz2, a.rdz2);
    t = t + cdiv(a, mr * zz, re, a.rre);
  }
  delta = 0.5 * (D[q] + D[q + sy]);
  rr = rho * re;
  yr = a.fast ? 1.0 / rr : 0.0;
  vx = cdiv(a, 0.5 * (V[q + sx] - V[q - sx]), dx, a.rdx);
  vy = cdiv(a, 0.5 * (V[q + sy] - V[q - sy]), dy, a.rdy);
  uy = cdiv(a, 0.5 * (((U[q + sy] - U[q]) + U[q - sx + sy]) - U[q - sx]), dy, a.rdy);
  phix = cdiv(a, 0.25 * (((P[q + sx] - P[q - sx]) + P[q + sx + sy]) - P[q - sx + sy]), dx, a.rdx);
  phiy = cdiv(a, P[q + sy] - P[q], dy, a.rdy);
  dxx = NS_DRR(c1 * delta * phix * (uy + vx));
  dyy = NS_DRR(c1 * delta * phiy * 2.0 * vy);
  t = (t + dxx) + dyy;
  if (kThree) {
    vz = cdiv(a, 0.5 * (V[q + sz] - V[q - sz]), dz, a.rdz);
    wy = cdiv(a, 0.5 * (((W[q + sy] - W[q]) + W[q + sy - sz]) - W[q - sz]), dy, a.rdy);
    phiz = cdiv(a, 0.25 * (((P[q + sy + sz] - P[q + sy - sz]) + P[q + sz]) - P[q - sz]), dz, a.rdz);
    dzz = NS_DRR(c1 * delta * phiz * (wy + vz));
    t = t + dzz;
  }
  t = t + a.gterm[1];
  if (sf) {
    curv = (CV[q] + CV[q + sy]) / 2.0;
    phiy = 0.5 * (N2[q] + N2[q + sy]);
    t = t - a.btn_sf * curv * delta * phiy / (a.we * rho);
  }
  TV[q] = t;
  if (!kThree) return;
  // ---- z: w at (i, j, k+1/2) ----
  rho = 0.5 * (R[q] + R[q + sz]);
  mu = 0.5 * (M[q] + M[q + sz]);
  mr = mu / rho;
  xx = cdiv(a, (W[q + sx] - 2.0 * W[q]) + W[q - sx], dx2, a.rdx2);
  yy = cdiv(a, (W[q + sy] - 2.0 * W[q]) + W[q - sy], dy2, a.rdy2);
  zz = cdiv(a, (W[q + sz] - 2.0 * W[q]) + W[q - sz], dz2, a.rdz2);
  t = (cdiv(a, mr * xx, re, a.rre) + cdiv(a, mr * yy, re, a.rre)) + cdiv(a, mr * zz, re, a.rre);
  delta = 0.5 * (D[q] + D[q + sz]);
  rr = rho * re;
  yr = a.fast ? 1.0 / rr : 0.0;
  wx = cdiv(a, 0.5 * (W[q + sx] - W[q - sx]), dx, a.rdx);
  wy = cdiv(a, 0.5 * (W[q + sy] - W[q - sy]), dy, a.rdy);
  wz = cdiv(a, 0.5 * (W[q + sz] - W[q - sz]), dz, a.rdz);
  uz = cdiv(a, 0.5 * (((U[q + sz] - U[q]) + U[q - sx + sz]) - U[q - sx]), dz, a.rdz);
  vz = cdiv(a, 0.5 * (((V[q + sz] - V[q]) + V[q - sy + sz]) - V[q - sy]), dz, a.rdz);
  phix = cdiv(a, 0.25 * (((P[q + sx + sz] - P[q - sx + sz]) + P[q + sx]) - P[q - sx]), dx, a.rdx);
  phiy = cdiv(a, 0.25 * (((P[q + sy + sz] - P[q - sy + sz]) + P[q + sy]) - P[q - sy]), dy, a.rdy);
  phiz = cdiv(a, P[q + sz] - P[q], dz, a.rdz);
  dxx = NS_DRR(c1 * delta * phix * (uz + wx));
  dyy = NS_DRR(c1 * delta * phiy * (vz + wy));
  dzz = NS_DRR(c1 * delta * phiz * 2.0 * wz);
  t = ((t + dxx) + dyy) + dzz;
  t = t + a.gterm[2];
  if (sf) {
    curv = (CV[q] + CV[q + sz]) / 2.0;
    phiz = 0.5 * (N3[q] + N3[q + sz]);
    t = t - a.btn_sf * curv * delta * phiz / (a.we * rho);
  }
  TW[q] = t;
#undef NS_DRR
}

// (a + |a|) m + (a - |a|) p: the upwind choice of ns_ab_adv_source_sec
__device__ __forceinline__ double ns_upwind(double a, double m, double p) {
  return (a + fabs(a)) * m + (a - fabs(a)) * p;
}

// -(sum over axes of upwind(a_d, one-sided differences of f along d)/2)
template <bool kThree>
__device__ __forceinline__ double ns_adv(const NsArgs& A, const double* __restrict__ f, int64_t q,
                                         const double (&a)[3]) {
  const int64_t st[3] = {1, A.sy, A.sz};
  const double h[3] = {A.dx, A.dy, A.dz};
  const double rh[3] = {A.rdx, A.rdy, A.rdz};
  double src = 0.0;
#pragma unroll
  for (int d = 0; d < (kThree ? 3 : 2); ++d) {
    const int64_t s = st[d];
    const double fp = cdiv(A, 0.5 * ((-f[q + 2 * s] + 4.0 * f[q + s]) - 3.0 * f[q]), h[d], rh[d]);
    const double fm = cdiv(A, 0.5 * ((f[q - 2 * s] - 4.0 * f[q - s]) + 3.0 * f[q]), h[d], rh[d]);
    const double term = ns_upwind(a[d], fm, fp) / 2.0;
    src = d == 0 ? -term : src - term;
  }
  return src;
}

// ns_ab_adv_source_quick: -(sum over axes d of ah_d (s_d(q) - s_d(q - e_d))/h_d),
// s_d the QUICK face value along d from the old velocity f, chosen upwind by
// ah_d = the average of the advecting velocity T_d over q and q + e_c.
template <bool kThree>
__device__ __forceinline__ double ns_adv_quick(const NsArgs& A, const double* __restrict__ f,
                                               int64_t q, int64_t ec,
                                               const double* const (&T)[3]) {
  const int64_t st[3] = {1, A.sy, A.sz};
  const double h[3] = {A.dx, A.dy, A.dz};
  const double rh[3] = {A.rdx, A.rdy, A.rdz};
  double src = 0.0;
#pragma unroll
  for (int d = 0; d < (kThree ? 3 : 2); ++d) {
    const int64_t s = st[d];
    double sv[2], ah = 0.0;
#pragma unroll
    for (int m = 0; m < 2; ++m) {
      const int64_t pq = m == 0 ? q - s : q;
      const double av = 0.5 * (T[d][pq] + T[d][pq + ec]);
      sv[m] = av >= 0.0 ? ((-f[pq - s] + 6.0 * f[pq]) + 3.0 * f[pq + s]) / 8.0
                        : ((-f[pq + 2 * s] + 6.0 * f[pq + s]) + 3.0 * f[pq]) / 8.0;
      if (m == 1) ah = av;
    }
    const double term = cdiv(A, ah * (sv[1] - sv[0]), h[d], rh[d]);
    src = d == 0 ? -term : src - term;
  }
  return src;
}

template <bool kThree>
__global__ void __launch_bounds__(kNsBx * kNsBy)
    k_ns_advance(NsArgs a, const double* __restrict__ U, const double* __restrict__ V,
                 const double* __restrict__ W, const double* __restrict__ Ut,
                 const double* __restrict__ Vt, const double* __restrict__ Wt,
                 const double* __restrict__ TU, const double* __restrict__ TV,
                 const double* __restrict__ TW, const double* __restrict__ SUo,
                 const double* __restrict__ SVo, const double* __restrict__ SWo,
                 double* __restrict__ SU, double* __restrict__ SV, double* __restrict__ SW,
                 double* __restrict__ Un, double* __restrict__ Vn, double* __restrict__ Wn) {
  const int i = blockIdx.x * kNsBx + threadIdx.x + 1;
  const int j = blockIdx.y * kNsBy + threadIdx.y + 1;
  const int k = blockIdx.z + 1;
  if (i > a.nx || j > a.ny) return;
  const int64_t sx = 1, sy = a.sy, sz = a.sz;
  const int64_t q = ns_at(a, i, j, k);
  const double dt = a.dt;
  double c[3], src;
  // x: u at (i+1/2, j, k), advected by u and the averages of v (and w) there
  c[0] = Ut[q];
  c[1] = 0.25 * (((Vt[q] + Vt[q - sy]) + Vt[q + sx]) + Vt[q + sx - sy]);
  c[2] = kThree ? 0.25 * (((Wt[q] + Wt[q - sz]) + Wt[q + sx]) + Wt[q + sx - sz]) : 0.0;
  const double* const Tq[3] = {Ut, Vt, Wt};
  src = (a.scheme == 1 ? ns_adv_quick<kThree>(a, U, q, sx, Tq) : ns_adv<kThree>(a, U, q, c)) +
        TU[q];
  SU[q] = src;
  Un[q] = U[q] + dt * (1.5 * src - 0.5 * SUo[q]);
  // y: v at (i, j+1/2, k)
  c[0] = 0.25 * (((Ut[q] + Ut[q - sx]) + Ut[q + sy]) + Ut[q - sx + sy]);
  c[1] = Vt[q];
  c[2] = kThree ? 0.25 * (((Wt[q] + Wt[q - sz]) + Wt[q + sy]) + Wt[q + sy - sz]) : 0.0;
  src = (a.scheme == 1 ? ns_adv_quick<kThree>(a, V, q, sy, Tq) : ns_adv<kThree>(a, V, q, c)) +
        TV[q];
  SV[q] = src;
  Vn[q] = V[q] + dt * (1.5 * src - 0.5 * SVo[q]);
  if (!kThree) return;
  // z: w at (i, j, k+1/2)
  c[0] = 0.25 * (((Ut[q] + Ut[q - sx]) + Ut[q + sz]) + Ut[q - sx + sz]);
  c[1] = 0.25 * (((Vt[q] + Vt[q - sy]) + Vt[q + sz]) + Vt[q - sy + sz]);
  c[2] = Wt[q];
  src = (a.scheme == 1 ? ns_adv_quick<kThree>(a, W, q, sz, Tq) : ns_adv<kThree>(a, W, q, c)) +
        TW[q];
  SW[q] = src;
  Wn[q] = W[q] + dt * (1.5 * src - 0.5 * SWo[q]);
}

// One axis of velbc for padded index x of an axis with n interior cells.
// Low side (bc 1 or 2): staggered (the component normal to this axis)
// f(1-m) = s f(m-1) for m = 1..g, then f(0) = 0; cell-centred f(1-m) = s f(m).
// High side: staggered f(n+m) = s f(n-m), then f(n) = 0; cell-centred
// f(n+m) = s f(n+1-m).  s = -1 for bc 1 (no-slip), +1 for bc 2 (slip).
struct AxisMap {
  int src;
  bool touched, zero, neg;
};

__device__ __forceinline__ AxisMap velbc_axis(int x, int n, bool stag, int lo, int hi) {
  AxisMap m{x, false, false, false};
  const bool alo = lo == 1 || lo == 2, ahi = hi == 1 || hi == 2;
  if (alo && x <= 0) {
    m.touched = true;
    m.neg = lo == 1;
    if (stag) {
      m.zero = x == 0;
      m.src = -x;
    } else {
      m.src = 1 - x;
    }
  } else if (ahi && (stag ? x >= n : x > n)) {
    m.touched = true;
    m.neg = hi == 1;
    if (stag) {
      m.zero = x == n;
      m.src = 2 * n - x;
    } else {
      m.src = 2 * n + 1 - x;
    }
  }
  return m;
}

// One warp per padded row (j, k).  Rows on the y or z shell (for the
// component) are done whole; other rows only at their x ghosts and walls.
template <bool kThree>
__global__ void __launch_bounds__(256) k_velbc(NsArgs a, NsBc bc, double* U, double* V,
                                               double* W) {
  const int g = a.g;
  const int py = a.ny + 2 * g, pz = kThree ? a.nz + 2 * g : 1;
  const int rows = py * pz;
  const int lane = threadIdx.x & 31;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  double* F[3] = {U, V, W};
  for (int r = warp; r < rows; r += nwarps) {
    const int j = r % py + 1 - g;
    const int k = kThree ? r / py + 1 - g : 1;
#pragma unroll 1
    for (int c = 0; c < (kThree ? 3 : 2); ++c) {
      const AxisMap my = velbc_axis(j, a.ny, c == 1, bc.b[2], bc.b[3]);
      const AxisMap mz = kThree ? velbc_axis(k, a.nz, c == 2, bc.b[4], bc.b[5])
                                : AxisMap{k, false, false, false};
      const bool whole = my.touched || mz.touched;
      // x positions of the row: all of them, or the low ghosts (and wall)
      // 1-g..0 followed by the high ghosts (and wall) nx+1-stag..nx+g
      const int lo_cnt = g, hi_first = a.nx + (c == 0 ? 0 : 1), hi_cnt = a.nx + g - hi_first + 1;
      const int cnt = whole ? a.nx + 2 * g : lo_cnt + hi_cnt;
      double* f = F[c];
      for (int t = lane; t < cnt; t += 32) {
        const int i = whole ? t + 1 - g : (t < lo_cnt ? t + 1 - g : hi_first + (t - lo_cnt));
        const AxisMap mx = velbc_axis(i, a.nx, c == 0, bc.b[0], bc.b[1]);
        if (!(mx.touched || my.touched || mz.touched)) continue;
        double v = f[ns_at(a, mx.src, my.src, mz.src)];
        if (mx.touched) v = mx.zero ? 0.0 : (mx.neg ? -v : v);
        if (my.touched) v = my.zero ? 0.0 : (my.neg ? -v : v);
        if (mz.touched) v = mz.zero ? 0.0 : (mz.neg ? -v : v);
        f[ns_at(a, i, j, k)] = v;
      }
    }
  }
}

// max |now - tmp| (bit pattern, atomicMax) and sum (now - tmp)^2 over the
// interior loops, into R.result[kSlotMax] and R.result[kSlotSum].
template <bool kThree>
__global__ void __launch_bounds__(kRedThreads) k_ns_change(NsArgs a, const double* U,
                                                           const double* V, const double* W,
                                                           const double* Ut, const double* Vt,
                                                           const double* Wt, ReduceScratch R) {
  double acc[1] = {0.0};
  double mx = 0.0;
  const int rows = a.ny * a.nz;
  for (int row = blockIdx.x; row < rows; row += gridDim.x) {
    const int j = row % a.ny + 1, k = row / a.ny + 1;
    for (int i = threadIdx.x + 1; i <= a.nx; i += blockDim.x) {
      const int64_t q = ns_at(a, i, j, k);
      const double du = U[q] - Ut[q], dv = V[q] - Vt[q];
      mx = fmax(mx, fabs(du));
      mx = fmax(mx, fabs(dv));
      acc[0] += du * du;
      acc[0] += dv * dv;
      if (kThree) {
        const double dw = W[q] - Wt[q];
        mx = fmax(mx, fabs(dw));
        acc[0] += dw * dw;
      }
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_down_sync(0xffffffffu, mx, o));
  if ((threadIdx.x & 31) == 0)
    atomicMax(reinterpret_cast<unsigned long long*>(R.result + kSlotMax),
              (unsigned long long)__double_as_longlong(mx));
  grid_sum_finish<1>(acc, R, kSlotSum);
}

// ls_funs + rho_mu over the whole padded box ("Two phase flows/newOpenMP/2D/
// src/interface_solver/others.f90:1-61"): x = phi/ls_wid, heavy = 1 above
// 1 - 1e-12, 0 below -1 + 1e-12, else (1 + x + sin(pi x)/pi)/2 clipped to
// [0, 1]; delta = (1 + cos(pi x))/(2 ls_wid) inside the band, else 0;
// rho = heavy + rho_12 (1 - heavy), mu = heavy + mu_12 (1 - heavy).
// Arrays at element (1,1,1); CUDA's sin and cos.
__global__ void __launch_bounds__(256) k_ns_rho_mu(NsArgs a, const double* __restrict__ phi,
                                                   double ls_wid, double rho_12,
                                                   double* __restrict__ rho,
                                                   double* __restrict__ mu,
                                                   double* __restrict__ delta) {
  const int g = a.g;
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1 - g;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1 - g;
  const int k = (a.nz > 1 ? (int)blockIdx.z + 1 - g : 1);
  if (i > a.nx + g || j > a.ny + g) return;
  const int64_t q = ns_at(a, i, j, k);
  const double pi = 3.141592653589793;
  const double eps = 1.0e-12;
  const double x = phi[q] / ls_wid;
  double heavy, hp;
  if (x > 1.0 - eps) {
    heavy = 1.0;
    hp = 0.0;
  } else if (x < -1.0 + eps) {
    heavy = 0.0;
    hp = 0.0;
  } else {
    heavy = 0.5 * (1.0 + x + sin(pi * x) / pi);
    hp = 0.5 * (1.0 + cos(pi * x)) / ls_wid;
  }
  heavy = fmax(fmin(heavy, 1.0), 0.0);
  if (rho) rho[q] = heavy + rho_12 * (1.0 - heavy);
  if (mu) mu[q] = heavy + a.mu_12 * (1.0 - heavy);
  if (delta) delta[q] = hp;
}

// ibm_bc's forcing ("Two phase flows/newOpenMP/3D+IBM/src/ns_solver/
// ns_solvers.f90:150-211") on the interior faces: with s the face average of
// the cell solid fraction, u = (1 - s) u, v = (1 - s) v (2D: the last
// component takes the body velocity), w = (1 - s) w + s w_body.
template <bool kThree>
__global__ void __launch_bounds__(kNsBx * kNsBy)
    k_ns_ibm(NsArgs a, const double* __restrict__ S, double w_body, double* U, double* V,
             double* W) {
  const int i = blockIdx.x * kNsBx + threadIdx.x + 1;
  const int j = blockIdx.y * kNsBy + threadIdx.y + 1;
  const int k = blockIdx.z + 1;
  if (i > a.nx || j > a.ny) return;
  const int64_t q = ns_at(a, i, j, k);
  double s = 0.5 * (S[q] + S[q + 1]);
  U[q] = (1.0 - s) * U[q];
  s = 0.5 * (S[q] + S[q + a.sy]);
  V[q] = kThree ? (1.0 - s) * V[q] : (1.0 - s) * V[q] + s * w_body;
  if (!kThree) return;
  s = 0.5 * (S[q] + S[q + a.sz]);
  W[q] = (1.0 - s) * W[q] + s * w_body;
}

dim3 ns_grid(const NsArgs& a) {
  return dim3((unsigned)((a.nx + kNsBx - 1) / kNsBx), (unsigned)((a.ny + kNsBy - 1) / kNsBy),
              (unsigned)a.nz);
}

}  // namespace

void launch_ns_diffusion(cudaStream_t s, const NsArgs& a, const double* const vel[3],
                         const double* rho, const double* mu, const double* delta,
                         const double* phi, const double* const nrm[3], const double* curv,
                         double* const out[3]) {
  const dim3 block(kNsBx, kNsBy);
  if (a.nz > 1)
    k_ns_diffusion<true><<<ns_grid(a), block, 0, s>>>(a, vel[0], vel[1], vel[2], rho, mu, delta,
                                                      phi, nrm[0], nrm[1], nrm[2], curv, out[0],
                                                      out[1], out[2]);
  else
    k_ns_diffusion<false><<<ns_grid(a), block, 0, s>>>(a, vel[0], vel[1], nullptr, rho, mu,
                                                       delta, phi, nrm[0], nrm[1], nullptr, curv,
                                                       out[0], out[1], nullptr);
}

void launch_ns_advance(cudaStream_t s, const NsArgs& a, const double* const old[3],
                       const double* const tmp[3], const double* const diff[3],
                       const double* const src_old[3], double* const src[3],
                       double* const now[3]) {
  const dim3 block(kNsBx, kNsBy);
  if (a.nz > 1)
    k_ns_advance<true><<<ns_grid(a), block, 0, s>>>(
        a, old[0], old[1], old[2], tmp[0], tmp[1], tmp[2], diff[0], diff[1], diff[2], src_old[0],
        src_old[1], src_old[2], src[0], src[1], src[2], now[0], now[1], now[2]);
  else
    k_ns_advance<false><<<ns_grid(a), block, 0, s>>>(
        a, old[0], old[1], nullptr, tmp[0], tmp[1], nullptr, diff[0], diff[1], nullptr,
        src_old[0], src_old[1], nullptr, src[0], src[1], nullptr, now[0], now[1], nullptr);
}

void launch_velbc(cudaStream_t s, const NsArgs& a, const NsBc& bc, double* const vel[3]) {
  const int pz = a.nz > 1 ? a.nz + 2 * a.g : 1;
  const long rows = (long)(a.ny + 2 * a.g) * pz;
  const unsigned blocks = (unsigned)std::min<long>((rows + 7) / 8, 152L * 16);
  if (a.nz > 1)
    k_velbc<true><<<blocks, 256, 0, s>>>(a, bc, vel[0], vel[1], vel[2]);
  else
    k_velbc<false><<<blocks, 256, 0, s>>>(a, bc, vel[0], vel[1], nullptr);
}

void launch_ns_change(cudaStream_t s, const NsArgs& a, const double* const now[3],
                      const double* const tmp[3], const ReduceScratch& R) {
  cudaMemsetAsync(R.result + kSlotMax, 0, sizeof(double), s);
  const int blocks = std::min(reduce_blocks_for((size_t)a.ny * a.nz), R.max_blocks);
  if (a.nz > 1)
    k_ns_change<true><<<blocks, kRedThreads, 0, s>>>(a, now[0], now[1], now[2], tmp[0], tmp[1],
                                                     tmp[2], R);
  else
    k_ns_change<false><<<blocks, kRedThreads, 0, s>>>(a, now[0], now[1], nullptr, tmp[0], tmp[1],
                                                      nullptr, R);
}

void launch_ns_rho_mu(cudaStream_t s, const NsArgs& a, const double* phi, double ls_wid,
                      double rho_12, double* rho, double* mu, double* delta) {
  const dim3 block(32, 8);
  const dim3 grid((unsigned)((a.nx + 2 * a.g + 31) / 32), (unsigned)((a.ny + 2 * a.g + 7) / 8),
                  (unsigned)(a.nz > 1 ? a.nz + 2 * a.g : 1));
  k_ns_rho_mu<<<grid, block, 0, s>>>(a, phi, ls_wid, rho_12, rho, mu, delta);
}

void launch_ns_ibm(cudaStream_t s, const NsArgs& a, const double* solid, double w_body,
                   double* const vel[3]) {
  const dim3 block(kNsBx, kNsBy);
  if (a.nz > 1)
    k_ns_ibm<true><<<ns_grid(a), block, 0, s>>>(a, solid, w_body, vel[0], vel[1], vel[2]);
  else
    k_ns_ibm<false><<<ns_grid(a), block, 0, s>>>(a, solid, w_body, vel[0], vel[1], nullptr);
}

}  // namespace gbmg
