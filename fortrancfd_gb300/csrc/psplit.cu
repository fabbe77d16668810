// Pressure-split projection (sm_103a): the source and the velocity
// correction of the DomainDecomposition solver's pressure step
// ("DomainDecomposition/3D/src/ns_solver/ns_ppe_mg_solver.f90").  There the
// variable-density pressure equation is split so that the multigrid only ever
// sees the constant-coefficient Laplacian:
//     lap p = rho_12 div(u*)/dt + div((1 - rho_12 beta) grad p^)
// with beta = 2/(rho_i + rho_nb) on a face, rho_12 the density ratio and p^
// the extrapolated pressure, followed by
//     u_f -= dt [ (1/rho_12) dp/h + (beta_f - 1/rho_12) dp^/h ].
// The arithmetic is the reference's, term for term and in its order
// (ppe_mg_solver_init :62-136, ppe_mg_solver_src :138-221, ppe_mg_correction
// :223-276), with the zero-gradient ghosts of job_bc at the walls; products
// that precede an addition are rounded on their own (no fused multiply-add)
// so the results match the FP64 oracle bit for bit.  Divisions by a power-of-
// two spacing are products with its exact reciprocal.
#include <cmath>

#include "dword.cuh"
#include <algorithm>

#include "gbmg_internal.h"

namespace gbmg {

namespace {

inline unsigned cdiv(size_t a, unsigned b) { return (unsigned)((a + b - 1) / b); }

__device__ __forceinline__ double over(double x, double h, double ih, bool pow2) {
  return pow2 ? x * ih : x / h;
}

// coe of one face: (1 - 2 rho_12/(rho_i + rho_nb))/h^2
__device__ __forceinline__ double split_coe(double two_r12, double ra, double rb, double h2) {
  return __ddiv_rn(__dsub_rn(1.0, __ddiv_rn(two_r12, __dadd_rn(ra, rb))), h2);
}

__global__ void __launch_bounds__(256) k_psplit_rhs(int nx, int ny, int nz,
                                                    const double* __restrict__ rho, Strided u,
                                                    Strided v, Strided w,
                                                    const double* __restrict__ ph, double rho12,
                                                    double3 h, double3 ih, double3 h2, int pow2,
                                                    double dt, double* __restrict__ src) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i >= nx || j >= ny) return;
  const bool three = nz > 1;
  const size_t sz = (size_t)nx * ny;
  const size_t q = (size_t)k * sz + (size_t)j * nx + i;
  // walls: the ghost is a copy of the cell
  const size_t qr = i < nx - 1 ? q + 1 : q, ql = i > 0 ? q - 1 : q;
  const size_t qf = j < ny - 1 ? q + nx : q, qb = j > 0 ? q - nx : q;
  const size_t qu = k < nz - 1 ? q + sz : q, qd = k > 0 ? q - sz : q;
  const double two_r12 = 2.0 * rho12;
  const double rc = rho[q];
  const double r = split_coe(two_r12, rc, rho[qr], h2.x);
  const double l = split_coe(two_r12, rc, rho[ql], h2.x);
  const double f = split_coe(two_r12, rc, rho[qf], h2.y);
  const double b = split_coe(two_r12, rc, rho[qb], h2.y);
  double up = 0.0, dn = 0.0, c;
  if (three) {
    up = split_coe(two_r12, rc, rho[qu], h2.z);
    dn = split_coe(two_r12, rc, rho[qd], h2.z);
    c = -(((((r + l) + f) + b) + up) + dn);
  } else {
    c = -(((r + l) + f) + b);
  }
  const int64_t fu = i + j * u.sy + k * u.sz;
  const int64_t fv = i + j * v.sy + k * v.sz;
  double d = __dadd_rn(over(u.data[fu + 1] - u.data[fu], h.x, ih.x, pow2 & 1),
                       over(v.data[fv + v.sy] - v.data[fv], h.y, ih.y, pow2 & 2));
  if (three) {
    const int64_t fw = i + j * w.sy + k * w.sz;
    d = __dadd_rn(d, over(w.data[fw + w.sz] - w.data[fw], h.z, ih.z, pow2 & 4));
  }
  d = d / dt;
  double s = __dadd_rn(__dmul_rn(d, rho12), __dmul_rn(c, ph[q]));
  s = __dadd_rn(s, __dmul_rn(r, ph[qr]));
  s = __dadd_rn(s, __dmul_rn(l, ph[ql]));
  s = __dadd_rn(s, __dmul_rn(f, ph[qf]));
  s = __dadd_rn(s, __dmul_rn(b, ph[qb]));
  if (three) {
    s = __dadd_rn(s, __dmul_rn(up, ph[qu]));
    s = __dadd_rn(s, __dmul_rn(dn, ph[qd]));
  }
  src[q] = s;
}

// one face's update: u -= dt ((1/rho_12) dp/h + (2/(ra+rb) - 1/rho_12) dph/h)
__device__ __forceinline__ double split_face(double uf, double ra, double rb, double dp,
                                             double dph, double inv_r12, double hh, double ihh,
                                             bool pow2, double dt) {
  double s = over(__dmul_rn(inv_r12, dp), hh, ihh, pow2);
  s = __dadd_rn(s, over(__dmul_rn(__dsub_rn(2.0 / __dadd_rn(ra, rb), inv_r12), dph), hh, ihh,
                        pow2));
  return __dsub_rn(uf, __dmul_rn(s, dt));
}

// Each cell corrects its high faces (the reference's u(i) on face i+1/2);
// wall faces see zero differences through the ghosts and are left as given.
__global__ void __launch_bounds__(256) k_psplit_correct(
    int nx, int ny, int nz, const double* __restrict__ rho, const double* __restrict__ p,
    const double* __restrict__ ph, double inv_r12, double3 h, double3 ih, int pow2, double dt,
    double* u, int64_t usy, int64_t usz, double* v, int64_t vsy, int64_t vsz, double* w,
    int64_t wsy, int64_t wsz) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i >= nx || j >= ny) return;
  const size_t sz = (size_t)nx * ny;
  const size_t q = (size_t)k * sz + (size_t)j * nx + i;
  if (i < nx - 1) {
    double* uf = u + (i + 1) + j * usy + k * usz;
    *uf = split_face(*uf, rho[q], rho[q + 1], p[q + 1] - p[q], ph[q + 1] - ph[q], inv_r12, h.x,
                     ih.x, pow2 & 1, dt);
  }
  if (j < ny - 1) {
    double* vf = v + i + (j + 1) * vsy + k * vsz;
    *vf = split_face(*vf, rho[q], rho[q + nx], p[q + nx] - p[q], ph[q + nx] - ph[q], inv_r12, h.y,
                     ih.y, pow2 & 2, dt);
  }
  if (k < nz - 1 && w) {
    double* wf = w + i + j * wsy + (k + 1) * wsz;
    *wf = split_face(*wf, rho[q], rho[q + sz], p[q + sz] - p[q], ph[q + sz] - ph[q], inv_r12,
                     h.z, ih.z, pow2 & 4, dt);
  }
}

// Face coefficients of the constant-coefficient Laplacian: 1/h^2 inside,
// 0 on the low wall faces (the storage convention of k_face_coef).
__global__ void __launch_bounds__(256) k_face_const(int nx, int ny, int nz, double3 c,
                                                   double* cx, double* cy, double* cz,
                                                   float* cx32, float* cy32, float* cz32,
                                                   float2* cxw, float2* cyw, float2* czw) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i >= nx || j >= ny) return;
  const size_t q = ((size_t)k * ny + j) * nx + i;
  const double vx = i > 0 ? c.x : 0.0, vy = j > 0 ? c.y : 0.0, vz = k > 0 ? c.z : 0.0;
  cx[q] = vx;
  cy[q] = vy;
  cz[q] = vz;
  if (cx32) {
    cx32[q] = (float)vx;
    cy32[q] = (float)vy;
    cz32[q] = (float)vz;
  }
  if (cxw) {
    const double vv[3] = {vx, vy, vz};
    float2* o[3] = {cxw, cyw, czw};
    for (int a = 0; a < 3; ++a) {
      const dw d = dw_from_double_int(vv[a]);
      o[a][q] = make_float2(d.hi, d.lo);
    }
  }
}

bool pow2_of(double v) {
  int e;
  return v > 0.0 && std::frexp(v, &e) == 0.5;
}

int pow2_mask(double dx, double dy, double dz) {
  return (pow2_of(dx) ? 1 : 0) | (pow2_of(dy) ? 2 : 0) | (pow2_of(dz) ? 4 : 0);
}

dim3 grid3(int nx, int ny, int nz) { return dim3(cdiv((size_t)nx, 32), cdiv((size_t)ny, 8), (unsigned)nz); }

// ph = w p + (1 - w) ph, the driver's new p^ after a stagnating cycle
// ("DomainDecomposition/3D/src/ns_solver/ns_ppe_mg_solver.f90:136-150"), in
// that operation order (products rounded, then the sum)
__global__ void k_guess_update(const double* __restrict__ p, double* __restrict__ ph, size_t n,
                               double w) {
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n;
       q += (size_t)gridDim.x * blockDim.x)
    ph[q] = __dadd_rn(__dmul_rn(w, p[q]), __dmul_rn(1.0 - w, ph[q]));
}

}  // namespace

void launch_psplit_rhs(cudaStream_t s, int nx, int ny, int nz, const double* rho, Strided u,
                       Strided v, Strided w, const double* ph, double rho12, double dx, double dy,
                       double dz, double dt, double* src) {
  k_psplit_rhs<<<grid3(nx, ny, nz), dim3(32, 8), 0, s>>>(
      nx, ny, nz, rho, u, v, w, ph, rho12, make_double3(dx, dy, dz),
      make_double3(1.0 / dx, 1.0 / dy, 1.0 / dz), make_double3(dx * dx, dy * dy, dz * dz),
      pow2_mask(dx, dy, dz), dt, src);
}

void launch_guess_update(cudaStream_t s, const double* p, double* ph, size_t n, double w) {
  k_guess_update<<<(unsigned)std::min<size_t>((n + 255) / 256, 152 * 16), 256, 0, s>>>(p, ph, n, w);
}

void launch_psplit_correct(cudaStream_t s, int nx, int ny, int nz, const double* rho,
                           const double* p, const double* ph, double rho12, double dx, double dy,
                           double dz, double dt, double* u, int64_t usy, int64_t usz, double* v,
                           int64_t vsy, int64_t vsz, double* w, int64_t wsy, int64_t wsz) {
  k_psplit_correct<<<grid3(nx, ny, nz), dim3(32, 8), 0, s>>>(
      nx, ny, nz, rho, p, ph, 1.0 / rho12, make_double3(dx, dy, dz),
      make_double3(1.0 / dx, 1.0 / dy, 1.0 / dz), pow2_mask(dx, dy, dz), dt, u, usy, usz, v, vsy,
      vsz, w, wsy, wsz);
}

void launch_face_const(cudaStream_t s, int nx, int ny, int nz, double dx2, double dy2, double dz2,
                       double* cx, double* cy, double* cz, float* const* c32, float2* const* cw) {
  k_face_const<<<grid3(nx, ny, nz), dim3(32, 8), 0, s>>>(
      nx, ny, nz, make_double3(1.0 / dx2, 1.0 / dy2, 1.0 / dz2), cx, cy, cz,
      c32 ? c32[0] : nullptr, c32 ? c32[1] : nullptr, c32 ? c32[2] : nullptr,
      cw ? cw[0] : nullptr, cw ? cw[1] : nullptr, cw ? cw[2] : nullptr);
}

}  // namespace gbmg
