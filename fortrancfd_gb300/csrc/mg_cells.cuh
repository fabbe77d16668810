// Per-cell bodies of the multigrid kernels (sm_103a), shared by the
// one-launch-per-step kernels of kernels_mg.cu and the one-block bottom of the
// cycle (subcycle.cu), so both do the same arithmetic in the same order.
// The cycle restated is the reference's ("DomainDecomposition/3D/src/
// others/multigrid_solver.f90": multigrid_relax :1-49, multigrid_restriction
// :51-90, multigrid_prolongation :106-160, multigrid_residual :162-222) on the
// variable-coefficient operator of ppe_sor_init.
#pragma once

#include <type_traits>

#include "gbmg_internal.h"

namespace gbmg {
namespace cells {

// A global load; kCg reads past L1 (ld.global.cg), for data that other blocks
// of the same kernel rewrite between phases (L1 is not coherent across SMs).
template <bool kCg, typename V>
__device__ __forceinline__ V ldc(const V* p) {
  if constexpr (kCg) return __ldcg(p);
  else return *p;
}

template <typename T> struct Vec2;
template <> struct Vec2<float> { using type = float2; };
template <> struct Vec2<double> { using type = double2; };

// Neighbour sum s = sum_f coe_f p_nb and diagonal d = sum_f coe_f of cell
// (i,j,k), accumulated in the order x-, x+, y-, y+, z-, z+.
template <typename T, bool kCg = false>
__device__ __forceinline__ void stencil(const LevelView<T>& L, const T* __restrict__ p, int i,
                                        int j, int k, size_t q, T& s, T& d) {
  const size_t sy = (size_t)L.nx, sz = (size_t)L.nx * L.ny;
  T c;
  s = T(0);
  d = T(0);
  if (i > 0) { c = L.cx[q]; s += c * ldc<kCg>(p + q - 1); d += c; }
  if (i < L.nx - 1) { c = L.cx[q + 1]; s += c * ldc<kCg>(p + q + 1); d += c; }
  if (j > 0) { c = L.cy[q]; s += c * ldc<kCg>(p + q - sy); d += c; }
  if (j < L.ny - 1) { c = L.cy[q + sy]; s += c * ldc<kCg>(p + q + sy); d += c; }
  if (k > 0) { c = L.cz[q]; s += c * ldc<kCg>(p + q - sz); d += c; }
  if (k < L.nz - 1) { c = L.cz[q + sz]; s += c * ldc<kCg>(p + q + sz); d += c; }
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
  const auto acc = [&](T cc, T pn) {
    if constexpr (std::is_same<T, float>::value) {
      rho_acc32(cc, pn, s, d);
    } else {
      s += cc * pn;
      d += cc;
    }
  };
  if (i > 0) { c = rho_face(L.kx, rc, r[q - 1]); acc(c, p[q - 1]); }
  if (i < L.nx - 1) { c = rho_face(L.kx, rc, r[q + 1]); acc(c, p[q + 1]); }
  if (j > 0) { c = rho_face(L.ky, rc, r[q - sy]); acc(c, p[q - sy]); }
  if (j < L.ny - 1) { c = rho_face(L.ky, rc, r[q + sy]); acc(c, p[q + sy]); }
  if (k > 0) { c = rho_face(L.kz, rc, r[q - sz]); acc(c, p[q - sz]); }
  if (k < L.nz - 1) { c = rho_face(L.kz, rc, r[q + sz]); acc(c, p[q + sz]); }
}

// The diagonal sum_f coe_f alone (same order as stencil_rho).
template <typename T>
__device__ __forceinline__ T diag_rho(const LevelView<T>& L, int i, int j, int k, size_t q) {
  const size_t sy = (size_t)L.nx, sz = (size_t)L.nx * L.ny;
  const T* __restrict__ r = L.rho;
  const T rc = r[q];
  T d = T(0);
  const auto add = [&](T cc) {
    if constexpr (std::is_same<T, float>::value) d = __fadd_rn(d, cc);
    else d += cc;
  };
  if (i > 0) add(rho_face(L.kx, rc, r[q - 1]));
  if (i < L.nx - 1) add(rho_face(L.kx, rc, r[q + 1]));
  if (j > 0) add(rho_face(L.ky, rc, r[q - sy]));
  if (j < L.ny - 1) add(rho_face(L.ky, rc, r[q + sy]));
  if (k > 0) add(rho_face(L.kz, rc, r[q - sz]));
  if (k < L.nz - 1) add(rho_face(L.kz, rc, r[q + sz]));
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
// kCg: read the level's unknown and right-hand side past L1 (ld.global.cg),
// for kernels in which other blocks rewrite them between phases.
template <typename T, bool kIdiag, bool kZero, bool kRho, bool kCg = false>
__device__ __forceinline__ void smooth_cell(const LevelView<T>& L, int i, int j, int k) {
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
    stencil<T, kCg>(L, L.sol, i, j, k, q, s, d);
  }
  if constexpr (kRho && std::is_same<T, float>::value) {
    L.sol[q] = rho_relax32(s, ldc<kCg>(L.src + q), d);
  } else {
    const T v = s - ldc<kCg>(L.src + q);
    if (kIdiag) L.sol[q] = v * L.idiag[q];
    else if (kRho) L.sol[q] = rho_update(v, d);
    else L.sol[q] = v / d;
  }
}


// Fused residual + restriction: coarse src = mean over the children of
// (src - A sol) on the fine level; coarse sol = 0.  One thread per coarse
// cell; the children are summed in the order z, y, x (the oracle's).
template <typename T, bool kRho, bool kCg = false>
__device__ __forceinline__ void restrict_cell(const LevelView<T>& F, const LevelView<T>& C, int I,
                                              int J, int K, int zero_sol) {
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
        const V2 p = ldc<kCg>(reinterpret_cast<const V2*>(F.sol + q));
        const V2 b = ldc<kCg>(reinterpret_cast<const V2*>(F.src + q));
        const bool xl = i0 > 0, xr = i0 + 2 < F.nx;
        const bool yl = j > 0, yr = j < F.ny - 1, zl = k > 0, zr = k < F.nz - 1;
        const T pl = xl ? ldc<kCg>(F.sol + q - 1) : T(0), pr = xr ? ldc<kCg>(F.sol + q + 2) : T(0);
        const V2 pym = yl ? ldc<kCg>(reinterpret_cast<const V2*>(F.sol + q - sy)) : zero2;
        const V2 pyp = yr ? ldc<kCg>(reinterpret_cast<const V2*>(F.sol + q + sy)) : zero2;
        const V2 pzm = zl ? ldc<kCg>(reinterpret_cast<const V2*>(F.sol + q - sz)) : zero2;
        const V2 pzp = zr ? ldc<kCg>(reinterpret_cast<const V2*>(F.sol + q + sz)) : zero2;
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
          else stencil<T, kCg>(F, F.sol, i, j, k, q, s, d);
          acc += ldc<kCg>(F.src + q) - (s - d * ldc<kCg>(F.sol + q));
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
template <typename T, bool kCg = false>
__device__ __forceinline__ void prolong_cell(const LevelView<T>& F, const LevelView<T>& C, int I,
                                             int J, int K) {
  using V2 = typename Vec2<T>::type;
  const size_t csy = (size_t)C.nx, csz = (size_t)C.nx * C.ny;
  const size_t cq = (size_t)K * csz + (size_t)J * csy + I;
  const T* e = C.sol;
  const T ec = ldc<kCg>(e + cq);
  T mx = T(0), my = T(0), mz = T(0);
  if (F.fx == 2)
    mx = T(0.5) * ((I < C.nx - 1 ? ldc<kCg>(e + cq + 1) : ec) - (I > 0 ? ldc<kCg>(e + cq - 1) : ec));
  if (F.fy == 2)
    my = T(0.5) * ((J < C.ny - 1 ? ldc<kCg>(e + cq + csy) : ec) -
                   (J > 0 ? ldc<kCg>(e + cq - csy) : ec));
  if (F.fz == 2)
    mz = T(0.5) * ((K < C.nz - 1 ? ldc<kCg>(e + cq + csz) : ec) -
                   (K > 0 ? ldc<kCg>(e + cq - csz) : ec));
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
        V2 cur = ldc<kCg>(pr);
        cur.x += v0;
        cur.y += v1;
        *pr = cur;
      } else {
        T v = ec;
        if (F.fy == 2) v += ty;
        if (F.fz == 2) v += tz;
        row[I] = ldc<kCg>(row + I) + v;
      }
    }
}


}  // namespace cells
}  // namespace gbmg
