// Interface normals and curvature by combined compact differences (CCD) on
// sm_103a: the reference's `curv` + `surface_norms` ("Two phase flows/
// newOpenMP/2D/src/interface_solver/others_normals.f90", 3D "…/3D+IBM/…")
// with the "ccd" scheme of lib/solver/ccd_solvers.f90 and the two-by-two
// block tridiagonal solver TWIN_DEC / TWIN_BKS of lib/solver/matrix_solver.f90.
//
// Every line of the ghost-padded box along an axis (L = n + 2g points, every
// other index over its padded range) is one block tridiagonal system for
// (f', f'').  Its matrix depends only on L and h, so k_ccd_decompose factors
// it once per axis (one thread, the reference's operations in order) into a
// table of 14 doubles per point that every line reads: the forward factors
// (row 1), the back-substitution factors (row 3), the diagonal blocks (row 2)
// and the block determinant with its IEEE reciprocal.  k_ccd_lines runs one
// line per thread: the right-hand side (asgn_src_ccd) is formed on the fly in
// the forward sweep from a sliding window of f, and the back substitution
// reads the swept values back.  Lines along y and z are coalesced (adjacent
// threads are adjacent in x); lines along x read with stride, served from L1.
// k_ccd_bc fills the ghost layers by zero-gradient copies (bc), k_curvature
// forms the curvature on the interior.
//
// FP64 in the reference's operand order, compiled with -fmad=false;
// quotients by h, h^2 and the block determinants come from correctly rounded
// reciprocals (fdiv.cuh), so the derivatives equal the oracle's bit for bit.
// The curvature's (|grad phi|^2 + 1e-12)^1.5 is formed as s * sqrt(s): sqrt is
// correctly rounded, so the power is within two roundings of exact (the
// reference's pow is within about one), at a fraction of pow's FP64 cost.
#include <algorithm>

#include "fdiv.cuh"
#include "gbmg_internal.h"
#include "reduce.cuh"

namespace gbmg {

namespace {

constexpr int kRec = 14;  // doubles per point of the factor table

// table layout per point i: A1 B1 AA1 BB1 | A3 B3 AA3 BB3 | A2 B2 AA2 BB2 | den rden
__global__ void k_ccd_decompose(int L, double h, double* __restrict__ work,
                                double* __restrict__ table) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  double* A = work;
  double* B = work + 3 * (size_t)L;
  double* AA = work + 6 * (size_t)L;
  double* BB = work + 9 * (size_t)L;
#define M_(X, r, i) X[((r) - 1) * (size_t)L + (i)]
  const int is = 0, ie = L - 1;
  // working_matrix_bc
  M_(A, 2, is) = 1.0; M_(B, 2, is) = 0.0; M_(AA, 2, is) = 0.0; M_(BB, 2, is) = 1.0;
  M_(A, 3, is) = 2.0; M_(B, 3, is) = -h; M_(AA, 3, is) = -(2.5 / h); M_(BB, 3, is) = 8.5;
  M_(A, 2, ie) = 1.0; M_(B, 2, ie) = 0.0; M_(AA, 2, ie) = 0.0; M_(BB, 2, ie) = 1.0;
  M_(A, 1, ie) = 2.0; M_(B, 1, ie) = h; M_(AA, 1, ie) = 2.5 / h; M_(BB, 1, ie) = 8.5;
  // working_matrix_init_ccd
  for (int i = is + 1; i <= ie - 1; ++i) {
    M_(A, 1, i) = 7.0 / 16.0; M_(A, 2, i) = 1.0; M_(A, 3, i) = 7.0 / 16.0;
    M_(B, 1, i) = h / 16.0; M_(B, 2, i) = 0.0; M_(B, 3, i) = -(h / 16.0);
    M_(AA, 1, i) = -(9.0 / 8.0 / h); M_(AA, 2, i) = 0.0; M_(AA, 3, i) = 9.0 / 8.0 / h;
    M_(BB, 1, i) = -(1.0 / 8.0); M_(BB, 2, i) = 1.0; M_(BB, 3, i) = -(1.0 / 8.0);
  }
  // TWIN_DEC
  M_(A, 1, is) = 0.0; M_(AA, 1, is) = 0.0; M_(A, 3, ie) = 0.0; M_(AA, 3, ie) = 0.0;
  M_(B, 1, is) = 0.0; M_(BB, 1, is) = 0.0; M_(B, 3, ie) = 0.0; M_(BB, 3, ie) = 0.0;
  for (int i = is + 1; i <= ie; ++i) {
    const double den = M_(A, 2, i - 1) * M_(BB, 2, i - 1) - M_(AA, 2, i - 1) * M_(B, 2, i - 1);
    double sc1 = -((M_(AA, 2, i - 1) * M_(B, 1, i) - M_(A, 1, i) * M_(BB, 2, i - 1)) / den);
    double sc2 = (M_(B, 1, i) * M_(A, 2, i - 1) - M_(B, 2, i - 1) * M_(A, 1, i)) / den;
    M_(A, 1, i) = sc1;
    M_(A, 2, i) = M_(A, 2, i) - (sc1 * M_(A, 3, i - 1) + sc2 * M_(AA, 3, i - 1));
    M_(B, 1, i) = sc2;
    M_(B, 2, i) = M_(B, 2, i) - (sc1 * M_(B, 3, i - 1) + sc2 * M_(BB, 3, i - 1));
    sc1 = -((M_(AA, 2, i - 1) * M_(BB, 1, i) - M_(AA, 1, i) * M_(BB, 2, i - 1)) / den);
    sc2 = (M_(BB, 1, i) * M_(A, 2, i - 1) - M_(B, 2, i - 1) * M_(AA, 1, i)) / den;
    M_(AA, 1, i) = sc1;
    M_(AA, 2, i) = M_(AA, 2, i) - (sc1 * M_(A, 3, i - 1) + sc2 * M_(AA, 3, i - 1));
    M_(BB, 1, i) = sc2;
    M_(BB, 2, i) = M_(BB, 2, i) - (sc1 * M_(B, 3, i - 1) + sc2 * M_(BB, 3, i - 1));
  }
  for (int i = 0; i < L; ++i) {
    double* t = table + (size_t)i * kRec;
    t[0] = M_(A, 1, i); t[1] = M_(B, 1, i); t[2] = M_(AA, 1, i); t[3] = M_(BB, 1, i);
    t[4] = M_(A, 3, i); t[5] = M_(B, 3, i); t[6] = M_(AA, 3, i); t[7] = M_(BB, 3, i);
    t[8] = M_(A, 2, i); t[9] = M_(B, 2, i); t[10] = M_(AA, 2, i); t[11] = M_(BB, 2, i);
    // the determinant of TWIN_BKS's diagonal block (the same products there)
    t[12] = M_(A, 2, i) * M_(BB, 2, i) - M_(AA, 2, i) * M_(B, 2, i);
    t[13] = 1.0 / t[12];
  }
#undef M_
}

__device__ __forceinline__ double qh(const CcdArgs& c, double x, double h, double rh) {
  return c.fast ? div_known(x, h, rh) : x / h;
}

// One line per thread.  Lines: line = i1 + n1 * i2, the line's first point
// at i1 s1 + i2 s2 from the box origin, points st apart.
__global__ void __launch_bounds__(128) k_ccd_lines(CcdBatch batch) {
  const int pass = blockIdx.y;
  const CcdArgs& c = batch.c[pass];
  const double* __restrict__ table = batch.table[pass];
  const double* __restrict__ f = batch.f[pass];
  double* __restrict__ S = batch.S[pass];
  double* __restrict__ SS = batch.SS[pass];
  const int line = blockIdx.x * blockDim.x + threadIdx.x;
  if (line >= c.n1 * c.n2) return;
  const int i1 = line % c.n1, i2 = line / c.n1;
  const int64_t base = (int64_t)i1 * c.s1 + (int64_t)i2 * c.s2;
  const int64_t st = c.st;
  const int L = c.L;
  const double* fl = f + base;
  double* Sl = S + base;
  double* SSl = SS + base;
  const double h = c.h, h2 = c.h2;
  // forward sweep with the right-hand side of asgn_src_ccd formed on the fly
  double fm = fl[0], fc = fl[st], fp = fl[2 * st];
  double s = qh(c, (-3.5 * fm + 4.0 * fc) - 0.5 * fp, h, c.rh);
  double ss = qh(c, ((34.0 / 3.0 * fm - 83.0 / 4.0 * fc) + 10.0 * fp) - 7.0 / 12.0 * fl[3 * st],
                 h2, c.rh2);
  Sl[0] = s;
  SSl[0] = ss;
  for (int i = 1; i < L - 1; ++i) {
    const double* t = table + (size_t)i * kRec;
    const double a1 = __ldg(t), b1 = __ldg(t + 1), aa1 = __ldg(t + 2), bb1 = __ldg(t + 3);
    if (i > 1) {
      fm = fc;
      fc = fp;
      fp = fl[(int64_t)(i + 1) * st];
    }
    double sn = qh(c, 15.0 / 16.0 * (-fm + fp), h, c.rh);
    double ssn = qh(c, (3.0 * fm - 6.0 * fc) + 3.0 * fp, h2, c.rh2);
    sn = sn - (a1 * s + b1 * ss);
    ssn = ssn - (aa1 * s + bb1 * ss);
    s = sn;
    ss = ssn;
    Sl[(int64_t)i * st] = s;
    SSl[(int64_t)i * st] = ss;
  }
  {
    const int i = L - 1;
    const double* t = table + (size_t)i * kRec;
    const double f0 = fl[(int64_t)i * st], f1 = fl[(int64_t)(i - 1) * st];
    const double f2 = fl[(int64_t)(i - 2) * st], f3 = fl[(int64_t)(i - 3) * st];
    double sn = -qh(c, (-3.5 * f0 + 4.0 * f1) - 0.5 * f2, h, c.rh);
    double ssn = qh(c, ((34.0 / 3.0 * f0 - 83.0 / 4.0 * f1) + 10.0 * f2) - 7.0 / 12.0 * f3, h2,
                    c.rh2);
    sn = sn - (__ldg(t) * s + __ldg(t + 1) * ss);
    ssn = ssn - (__ldg(t + 2) * s + __ldg(t + 3) * ss);
    s = sn;
    ss = ssn;
  }
  // back substitution (TWIN_BKS)
  double sol, sol2;
  {
    const double* t = table + (size_t)(L - 1) * kRec;
    const double a2 = __ldg(t + 8), b2 = __ldg(t + 9), aa2 = __ldg(t + 10), bb2 = __ldg(t + 11);
    const double den = __ldg(t + 12), rden = __ldg(t + 13);
    sol = -div_known_checked(b2 * ss - bb2 * s, den, rden);
    sol2 = div_known_checked(a2 * ss - aa2 * s, den, rden);
    Sl[(int64_t)(L - 1) * st] = sol;
    SSl[(int64_t)(L - 1) * st] = sol2;
  }
  for (int i = L - 2; i >= 0; --i) {
    const double* t = table + (size_t)i * kRec;
    const int64_t o = (int64_t)i * st;
    double si = Sl[o], ssi = SSl[o];
    si = si - (__ldg(t + 4) * sol + __ldg(t + 5) * sol2);
    ssi = ssi - (__ldg(t + 6) * sol + __ldg(t + 7) * sol2);
    const double a2 = __ldg(t + 8), b2 = __ldg(t + 9), aa2 = __ldg(t + 10), bb2 = __ldg(t + 11);
    const double den = __ldg(t + 12), rden = __ldg(t + 13);
    sol = -div_known_checked(b2 * ssi - bb2 * si, den, rden);
    sol2 = div_known_checked(a2 * ssi - aa2 * si, den, rden);
    Sl[o] = sol;
    SSl[o] = sol2;
  }
}

__device__ __forceinline__ int clampi(int x, int n) { return x < 1 ? 1 : (x > n ? n : x); }

// bc: every ghost value is the boundary value of its clamped index (the x,
// y, z passes of copies compose to that).  One warp per padded row; rows
// outside the interior in y or z are done whole, others at their x ghosts.
__global__ void __launch_bounds__(256) k_ccd_bc(NsArgs a, double* f0, double* f1, double* f2,
                                                double* f3) {
  const int g = a.g;
  const bool three = a.nz > 1;
  const int py = a.ny + 2 * g, pz = three ? a.nz + 2 * g : 1;
  const int rows = py * pz;
  const int lane = threadIdx.x & 31;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  double* F[4] = {f0, f1, f2, f3};
  for (int r = warp; r < rows; r += nwarps) {
    const int j = r % py + 1 - g;
    const int k = three ? r / py + 1 - g : 1;
    const bool whole = j < 1 || j > a.ny || (three && (k < 1 || k > a.nz));
    const int cnt = whole ? a.nx + 2 * g : 2 * g;
    const int jc = clampi(j, a.ny), kc = three ? clampi(k, a.nz) : 1;
    for (int t = lane; t < cnt; t += 32) {
      const int i = whole ? t + 1 - g : (t < g ? t + 1 - g : a.nx + 1 + (t - g));
      const int ic = clampi(i, a.nx);
      const int64_t src = (int64_t)(ic - 1) + (int64_t)(jc - 1) * a.sy + (int64_t)(kc - 1) * a.sz;
      const int64_t dst = (int64_t)(i - 1) + (int64_t)(j - 1) * a.sy + (int64_t)(k - 1) * a.sz;
#pragma unroll
      for (int c = 0; c < 4; ++c)
        if (F[c]) F[c][dst] = F[c][src];
    }
  }
}

// curv on the interior (others_normals.f90 curv): arrays at element (1,1,1)
template <bool kThree>
__global__ void __launch_bounds__(256) k_curvature(NsArgs a, const double* __restrict__ fx_,
                                                   const double* __restrict__ fy_,
                                                   const double* __restrict__ fz_,
                                                   const double* __restrict__ fxx,
                                                   const double* __restrict__ fyy,
                                                   const double* __restrict__ fzz,
                                                   const double* __restrict__ fxy,
                                                   const double* __restrict__ fxz,
                                                   const double* __restrict__ fyz,
                                                   double* __restrict__ curv) {
  const int i = blockIdx.x * 32 + threadIdx.x + 1;
  const int j = blockIdx.y * 8 + threadIdx.y + 1;
  const int k = blockIdx.z + 1;
  if (i > a.nx || j > a.ny) return;
  const int64_t q = (int64_t)(i - 1) + (int64_t)(j - 1) * a.sy + (int64_t)(k - 1) * a.sz;
  const double fx = fx_[q], fy = fy_[q];
  if (!kThree) {
    const double num = (fyy[q] * (fx * fx) + fxx[q] * (fy * fy)) - 2.0 * fxy[q] * fx * fy;
    const double sq = (fx * fx + fy * fy) + 1.0e-12;
    curv[q] = num / (sq * sqrt(sq));
  } else {
    const double fz = fz_[q];
    const double num = (((fyy[q] + fzz[q]) * (fx * fx) + (fxx[q] + fzz[q]) * (fy * fy)) +
                        (fxx[q] + fyy[q]) * (fz * fz)) -
                       2.0 * ((fxy[q] * fx * fy + fxz[q] * fx * fz) + fyz[q] * fy * fz);
    const double sq = ((fx * fx + fy * fy) + fz * fz) + 1.0e-12;
    curv[q] = num / (sq * sqrt(sq));
  }
}


// ls_funs at one value (others.f90:1-37): heavy and delta of x = phi/ls_wid
__device__ __forceinline__ void mp_funs(double phi, double ls_wid, double* heavy, double* delta) {
  const double pi = 3.141592653589793;
  const double x = phi / ls_wid;
  double h, hp;
  if (x > 1.0 - 1.0e-12) {
    h = 1.0;
    hp = 0.0;
  } else if (x < -1.0 + 1.0e-12) {
    h = 0.0;
    hp = 0.0;
  } else {
    h = 0.5 * (1.0 + x + sin(pi * x) / pi);
    hp = 0.5 * (1.0 + cos(pi * x)) / ls_wid;
  }
  *heavy = fmax(fmin(h, 1.0), 0.0);
  *delta = hp;
}

// mass_preserving_level_set's sums over the interior (ls_mv's mass and the
// lambda denominator): acc[0] = sum rho H dv, acc[1] = sum delta^2 |grad phi|
// (2 (1 - rho_12) H + rho_12) dv; |grad phi| from the compact gradient.
__global__ void __launch_bounds__(kRedThreads) k_mpls_sums(NsArgs a, const double* phi,
                                                           const double* gx, const double* gy,
                                                           const double* gz, double ls_wid,
                                                           double rho_12, double dv,
                                                           ReduceScratch R) {
  double acc[2] = {0.0, 0.0};
  const int rows = a.ny * a.nz;
  for (int row = blockIdx.x; row < rows; row += gridDim.x) {
    const int j = row % a.ny + 1, k = row / a.ny + 1;
    for (int i = threadIdx.x + 1; i <= a.nx; i += blockDim.x) {
      const int64_t q = (int64_t)(i - 1) + (int64_t)(j - 1) * a.sy + (int64_t)(k - 1) * a.sz;
      double heavy, delta;
      mp_funs(phi[q], ls_wid, &heavy, &delta);
      const double rho = heavy + rho_12 * (1.0 - heavy);
      acc[0] += rho * heavy * dv;
      if (!gx) continue;  // the mass alone
      const double g2 = gz ? (gx[q] * gx[q] + gy[q] * gy[q]) + gz[q] * gz[q]
                           : gx[q] * gx[q] + gy[q] * gy[q];
      const double grad = sqrt(g2);
      double plam = delta * delta * grad;
      plam = plam * (2.0 * (1.0 - rho_12) * heavy + rho_12) * a.dx * a.dy;
      if (gz) plam = plam * a.dz;
      acc[1] += plam;
    }
  }
  grid_sum_finish<2>(acc, R, kSlotSum);
}

// phi += lam delta |grad phi| on the interior (delta of the phi before)
__global__ void __launch_bounds__(256) k_mpls_update(NsArgs a, double* phi, const double* gx,
                                                     const double* gy, const double* gz,
                                                     double ls_wid, double lam) {
  const int i = blockIdx.x * 32 + threadIdx.x + 1;
  const int j = blockIdx.y * 8 + threadIdx.y + 1;
  const int k = blockIdx.z + 1;
  if (i > a.nx || j > a.ny) return;
  const int64_t q = (int64_t)(i - 1) + (int64_t)(j - 1) * a.sy + (int64_t)(k - 1) * a.sz;
  double heavy, delta;
  mp_funs(phi[q], ls_wid, &heavy, &delta);
  const double g2 = gz ? (gx[q] * gx[q] + gy[q] * gy[q]) + gz[q] * gz[q]
                       : gx[q] * gx[q] + gy[q] * gy[q];
  phi[q] = phi[q] + lam * delta * sqrt(g2);
}

// vof_wlic_solver's flux along axis ax at faces 0..n of that axis and rows
// 0..n of the others (the reference's is-1..ie ranges): the WLIC blend of the
// THINC flux (beta = 2.3) and the upwind flux by the normal's share, the
// normal being surface_norms2's central difference of phi at the clamped
// upwind cell (zero-gradient ghosts).  Arrays at element (1,1,1).
__global__ void __launch_bounds__(256) k_wlic_flux(NsArgs a, int ax, const double* __restrict__ vof,
                                                   const double* __restrict__ vel,
                                                   const double* __restrict__ phi,
                                                   double* __restrict__ flux) {
  const bool three = a.nz > 1;
  const int i = blockIdx.x * 32 + threadIdx.x;
  const int j = blockIdx.y * 8 + threadIdx.y;
  const int k = three ? (int)blockIdx.z : 1;
  if (i > a.nx || j > a.ny) return;
  const double eps = 1.0e-12, beta = 2.3;
  const double dt = a.dt;
  const double hs[3] = {a.dx, a.dy, a.dz};
  const int n[3] = {a.nx, a.ny, a.nz};
  const int64_t st[3] = {1, a.sy, a.sz};
  const int64_t q = (int64_t)(i - 1) + (int64_t)(j - 1) * a.sy + (int64_t)(k - 1) * a.sz;
  const double u = vel[q];
  int cc[3] = {i, j, k};
  double isgn = 1.0;
  if (!(u > 0.0)) {
    cc[ax] += 1;
    isgn = 0.0;
  }
  const int64_t qi = q + (cc[ax] - (ax == 0 ? i : (ax == 1 ? j : k))) * st[ax];
  const double f = vof[qi];
  double l;
  if (f > 1.0 - eps || f < eps) {
    l = f * u * dt;
  } else {
    const int cb = cc[ax] - 1 < 1 ? 1 : cc[ax] - 1;
    const int64_t qb = qi + (cb - cc[ax]) * st[ax];
    const double alpha = vof[qb] < vof[qi + st[ax]] ? 1.0 : -1.0;
    const double h = hs[ax];
    const double a1 = exp(beta * (2.0 * f - 1.0) / alpha);
    const double a3 = exp(beta);
    const double xc = 0.5 / beta * log((a3 * a3 - a1 * a3) / (a1 * a3 - 1.0));
    const double a4 = cosh(beta * ((isgn - u * dt / h) - xc));
    const double a5 = cosh(beta * (isgn - xc));
    int c[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) c[d] = cc[d] < 1 ? 1 : (cc[d] > n[d] ? n[d] : cc[d]);
    if (!three) c[2] = 1;
    const int64_t qc = (int64_t)(c[0] - 1) + (int64_t)(c[1] - 1) * a.sy + (int64_t)(c[2] - 1) * a.sz;
    double nrm[3];
    nrm[0] = 0.5 * (phi[qc + 1] - phi[qc - 1]) / a.dx;
    nrm[1] = 0.5 * (phi[qc + a.sy] - phi[qc - a.sy]) / a.dy;
    nrm[2] = three ? 0.5 * (phi[qc + a.sz] - phi[qc - a.sz]) / a.dz : 0.0;
    double w = three ? (fabs(nrm[0]) + fabs(nrm[1])) + fabs(nrm[2]) : fabs(nrm[0]) + fabs(nrm[1]);
    w = fabs(nrm[ax]) / w;
    l = 0.5 * (u * dt - alpha * h / beta * log(a4 / a5));
    l = l * w + (1.0 - w) * f * u * dt;
  }
  flux[q] = l;
}

// the cell update of one sweep (clipped to [0, 1] after the last sweep)
__global__ void __launch_bounds__(256) k_wlic_update(NsArgs a, int ax, int last, double* vof,
                                                     const double* __restrict__ vof_old,
                                                     const double* __restrict__ vel,
                                                     const double* __restrict__ flux) {
  const int i = blockIdx.x * 32 + threadIdx.x + 1;
  const int j = blockIdx.y * 8 + threadIdx.y + 1;
  const int k = blockIdx.z + 1;
  if (i > a.nx || j > a.ny) return;
  const double eps = 1.0e-12;
  const int64_t st = ax == 0 ? 1 : (ax == 1 ? a.sy : a.sz);
  const double h = ax == 0 ? a.dx : (ax == 1 ? a.dy : a.dz);
  const int64_t q = (int64_t)(i - 1) + (int64_t)(j - 1) * a.sy + (int64_t)(k - 1) * a.sz;
  double f = vof[q] - (flux[q] - flux[q - st]) / h + vof_old[q] * a.dt * (vel[q] - vel[q - st]) / h;
  if (last) {
    if (f < eps) f = 0.0;
    if (f > 1.0 - eps) f = 1.0;
  }
  vof[q] = f;
}
}  // namespace

void launch_ccd_decompose(cudaStream_t s, int L, double h, double* work, double* table) {
  k_ccd_decompose<<<1, 1, 0, s>>>(L, h, work, table);
}

void launch_ccd_lines(cudaStream_t s, const CcdBatch& b) {
  int lines = 0;
  for (int i = 0; i < b.n; ++i) lines = std::max(lines, b.c[i].n1 * b.c[i].n2);
  k_ccd_lines<<<dim3((unsigned)((lines + 127) / 128), (unsigned)b.n), 128, 0, s>>>(b);
}

void launch_ccd_bc(cudaStream_t s, const NsArgs& a, double* const f[4]) {
  const int pz = a.nz > 1 ? a.nz + 2 * a.g : 1;
  const long rows = (long)(a.ny + 2 * a.g) * pz;
  const unsigned blocks = (unsigned)std::min<long>((rows + 7) / 8, 152L * 16);
  k_ccd_bc<<<blocks, 256, 0, s>>>(a, f[0], f[1], f[2], f[3]);
}

void launch_curvature(cudaStream_t s, const NsArgs& a, const double* const d1[3],
                      const double* const d2[6], double* curv) {
  const dim3 block(32, 8);
  const dim3 grid((unsigned)((a.nx + 31) / 32), (unsigned)((a.ny + 7) / 8), (unsigned)a.nz);
  if (a.nz > 1)
    k_curvature<true><<<grid, block, 0, s>>>(a, d1[0], d1[1], d1[2], d2[0], d2[1], d2[2], d2[3],
                                             d2[4], d2[5], curv);
  else
    k_curvature<false><<<grid, block, 0, s>>>(a, d1[0], d1[1], nullptr, d2[0], d2[1], nullptr,
                                              d2[3], nullptr, nullptr, curv);
}

void launch_mpls_sums(cudaStream_t s, const NsArgs& a, const double* phi, const double* const g[3],
                      double ls_wid, double rho_12, double dv, const ReduceScratch& R) {
  const int blocks = std::min(reduce_blocks_for((size_t)a.ny * a.nz), R.max_blocks);
  k_mpls_sums<<<blocks, kRedThreads, 0, s>>>(a, phi, g[0], g[1], g[2], ls_wid, rho_12, dv, R);
}

void launch_mpls_update(cudaStream_t s, const NsArgs& a, double* phi, const double* const g[3],
                        double ls_wid, double lam) {
  const dim3 block(32, 8);
  const dim3 grid((unsigned)((a.nx + 31) / 32), (unsigned)((a.ny + 7) / 8), (unsigned)a.nz);
  k_mpls_update<<<grid, block, 0, s>>>(a, phi, g[0], g[1], g[2], ls_wid, lam);
}

void launch_wlic(cudaStream_t s, const NsArgs& a, int ax, double* vof, const double* vof_old,
                 const double* vel, const double* phi, double* flux) {
  const dim3 block(32, 8);
  const bool three = a.nz > 1;
  const dim3 gf((unsigned)((a.nx + 1 + 31) / 32), (unsigned)((a.ny + 1 + 7) / 8),
                (unsigned)(three ? a.nz + 1 : 1));
  k_wlic_flux<<<gf, block, 0, s>>>(a, ax, vof, vel, phi, flux);
  const dim3 gu((unsigned)((a.nx + 31) / 32), (unsigned)((a.ny + 7) / 8), (unsigned)a.nz);
  k_wlic_update<<<gu, block, 0, s>>>(a, ax, ax == (three ? 2 : 1), vof, vof_old, vel, flux);
}

}  // namespace gbmg
