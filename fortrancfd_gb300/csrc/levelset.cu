// Level-set transport on sm_103a: the advection step of the reference's
// interface solver, level_set_rk3_solver ("Two phase flows/newOpenMP/2D/src/
// interface_solver/level_set_rk3_solver.f90:1-186"; 3D "Two phase flows/
// newOpenMP/3D+IBM/src/interface_solver/level_set_rk3_solver.f90:1-215").
//
// phi_t + div(u phi) = 0 with the cell-centred velocity: the flux is split
// into u+ phi and u- phi (level_set_rk3_source_setup), each part is
// reconstructed at every face by WENO-JS (wenojs_flux_split, EPS = 1e-13) --
// u+ phi from the five cells left of the face, u- phi from the five cells
// right of it -- with zero-gradient ghosts (bc: an index outside the grid
// reads the nearest boundary cell), and three stages of SSP-RK3 in the
// reference's incremental form advance phi.  nz = 1 is the 2D solver.
//
// The faces are reconstructed once each (k_ls_faces, one thread per face,
// both split parts), then k_ls_stage forms L(phi) per cell in the
// reference's order and applies the stage.  All arithmetic is FP64 with every
// product rounded on its own (no fused multiply-add), so the results equal
// the FP64 oracle bit for bit.  GB300 runs FP64 at about 1/57 of its FP32
// rate and a face costs two reconstructions of about 20 divisions each, so
// these kernels are bound by the FP64 pipe, not by memory.
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <string>

#include "gbmg.h"
#include "fdiv.cuh"
#include "gbmg_internal.h"

namespace gbmg {

namespace {

__device__ __forceinline__ double dsq(double x) { return __dmul_rn(x, x); }
__device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dvd(double a, double b) { return __ddiv_rn(a, b); }
// Quotients by the run-time spacing come from its correctly rounded
// reciprocal without dividing (fdiv.cuh): the same doubles, cheaper where a
// kernel divides by h often (the redistancing gradient: 6 per cell and
// axis).  Divisions by literal constants and the WENO weights (a divisor
// used three times, whose reciprocal would cost a division of its own) stay
// IEEE divisions: measured faster so (advection step 96.5 against 106 ms).
__device__ __forceinline__ double by3(double a) { return dvd(a, 3.0); }
__device__ __forceinline__ double by6(double a) { return dvd(a, 6.0); }
__device__ __forceinline__ double by12(double a) { return dvd(a, 12.0); }
__device__ __forceinline__ double by4(double a) { return mul(a, 0.25); }  // exact

// value at face i+1/2 of g(i-2..i+2) = g0..g4, biased to the left
__device__ double weno_left(double g0, double g1, double g2, double g3, double g4, double eps) {
  const double b1 = add(mul(13.0, dsq(add(sub(g0, mul(2.0, g1)), g2))),
                        mul(3.0, dsq(add(sub(g0, mul(4.0, g1)), mul(3.0, g2)))));
  const double b2 = add(mul(13.0, dsq(add(sub(g1, mul(2.0, g2)), g3))), mul(3.0, dsq(sub(g1, g3))));
  const double b3 = add(mul(13.0, dsq(add(sub(g2, mul(2.0, g3)), g4))),
                        mul(3.0, dsq(add(sub(mul(3.0, g2), mul(4.0, g3)), g4))));
  const double a1 = dvd(1.0, dsq(add(eps, b1)));
  const double a2 = dvd(6.0, dsq(add(eps, b2)));
  const double a3 = dvd(3.0, dsq(add(eps, b3)));
  const double s = add(add(a1, a2), a3);
  const double w1 = dvd(a1, s), w2 = dvd(a2, s), w3 = dvd(a3, s);
  double v = mul(by3(w1), g0);
  v = sub(v, mul(by6(add(mul(7.0, w1), w2)), g1));
  v = add(v, mul(by6(add(add(mul(11.0, w1), mul(5.0, w2)), mul(2.0, w3))), g2));
  v = add(v, mul(by6(add(mul(2.0, w2), mul(5.0, w3))), g3));
  v = sub(v, mul(by6(w3), g4));
  return v;
}

// value at face i+1/2 of f(i-1..i+3) = f0..f4, biased to the right
__device__ double weno_right(double f0, double f1, double f2, double f3, double f4, double eps) {
  const double b3 = add(mul(13.0, dsq(add(sub(f0, mul(2.0, f1)), f2))),
                        mul(3.0, dsq(add(sub(f0, mul(4.0, f1)), mul(3.0, f2)))));
  const double b2 = add(mul(13.0, dsq(add(sub(f1, mul(2.0, f2)), f3))), mul(3.0, dsq(sub(f1, f3))));
  const double b1 = add(mul(13.0, dsq(add(sub(f2, mul(2.0, f3)), f4))),
                        mul(3.0, dsq(add(sub(mul(3.0, f2), mul(4.0, f3)), f4))));
  const double a1 = dvd(1.0, dsq(add(eps, b1)));
  const double a2 = dvd(6.0, dsq(add(eps, b2)));
  const double a3 = dvd(3.0, dsq(add(eps, b3)));
  const double s = add(add(a1, a2), a3);
  const double w1 = dvd(a1, s), w2 = dvd(a2, s), w3 = dvd(a3, s);
  double v = by6(mul(w3, add(add(-f0, mul(5.0, f1)), mul(2.0, f2))));
  v = add(v, by6(mul(w2, sub(add(mul(2.0, f1), mul(5.0, f2)), f3))));
  v = add(v, by6(mul(w1, add(sub(mul(11.0, f2), mul(7.0, f3)), mul(2.0, f4)))));
  return v;
}

__device__ __forceinline__ int clampi(int i, int n) { return i < 0 ? 0 : (i >= n ? n - 1 : i); }

struct LsGrid {
  int nx, ny, nz;
  double dx, dy, dz;
  double rdx, rdy, rdz;  // RN(1/dx) ...; fast = 1 when all three allow div_known
  int fast;
};

LsGrid ls_grid(const gbmg_grid& g) {
  LsGrid G{g.nx, g.ny, g.nz, g.dx, g.dy, g.dz, 1.0 / g.dx, 1.0 / g.dy, 1.0 / g.dz, 1};
  G.fast = fdiv_divisor_ok(g.dx) && fdiv_divisor_ok(g.dy) && fdiv_divisor_ok(g.dz);
  return G;
}

// a / h along an axis with the reciprocal from the grid
__device__ __forceinline__ double by_h(const LsGrid& g, double a, double h, double rh) {
  return g.fast ? div_known(a, h, rh) : __ddiv_rn(a, h);
}

// Faces of one axis: face f (0..n) is the reference's face i+1/2 with
// i = f - 1; ss1 = left-biased WENO of u+ phi, ss2 = right-biased of u- phi.
// The face arrays are laid out like cell arrays with n+1 entries along the
// axis.
__global__ void __launch_bounds__(256) k_ls_faces(LsGrid g, int axis, const double* __restrict__ phi,
                                                  const double* __restrict__ vel,
                                                  double* __restrict__ ss1,
                                                  double* __restrict__ ss2) {
  const int ex = g.nx + (axis == 0), ey = g.ny + (axis == 1), ez = g.nz + (axis == 2);
  const size_t nf = (size_t)ex * ey * ez;
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nf) return;
  const int a = (int)(t % ex);
  const size_t r = t / ex;
  const int b = (int)(r % ey), c = (int)(r / ey);
  // position of the face along the axis and the line through it
  const int f = axis == 0 ? a : (axis == 1 ? b : c);
  const int n = axis == 0 ? g.nx : (axis == 1 ? g.ny : g.nz);
  const size_t stride = axis == 0 ? 1 : (axis == 1 ? (size_t)g.nx : (size_t)g.nx * g.ny);
  const int i0 = axis == 0 ? 0 : a, j0 = axis == 1 ? 0 : b, k0 = axis == 2 ? 0 : c;
  const size_t base = ((size_t)k0 * g.ny + j0) * g.nx + i0;
  const int fi = f - 1;
  double gp[6], gm[6];  // u+ phi and u- phi of cells fi-2 .. fi+3
#pragma unroll
  for (int m = 0; m < 6; ++m) {
    const size_t q = base + (size_t)clampi(fi - 2 + m, n) * stride;
    const double u = vel[q], p = phi[q];
    gp[m] = mul(mul(0.5, add(u, fabs(u))), p);
    gm[m] = mul(mul(0.5, sub(u, fabs(u))), p);
  }
  const double eps = 1.0e-13;
  ss1[t] = weno_left(gp[0], gp[1], gp[2], gp[3], gp[4], eps);
  ss2[t] = weno_right(gm[1], gm[2], gm[3], gm[4], gm[5], eps);
}

// One stage: l = L(phi) per cell, then phi += src * dt with the stage's
// combination of l1, l2, l3 (level_set_rk3_solver).
__global__ void __launch_bounds__(256) k_ls_stage(LsGrid g, int stage, double dt,
                                                  const double* __restrict__ x1,
                                                  const double* __restrict__ x2,
                                                  const double* __restrict__ y1,
                                                  const double* __restrict__ y2,
                                                  const double* __restrict__ z1,
                                                  const double* __restrict__ z2, double* l1,
                                                  double* l2, double* phi) {
  const size_t n = (size_t)g.nx * g.ny * g.nz;
  const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const int i = (int)(q % g.nx);
  const size_t r = q / g.nx;
  const int j = (int)(r % g.ny), k = (int)(r / g.ny);
  // face indices: high face of the cell = low face + one step along the axis
  const size_t fx = ((size_t)k * g.ny + j) * (g.nx + 1) + i;
  const size_t fy = ((size_t)k * (g.ny + 1) + j) * g.nx + i;
  const size_t fz = ((size_t)k * g.ny + j) * g.nx + i;
  double d = sub(sub(add(x1[fx + 1], x2[fx + 1]), x1[fx]), x2[fx]);
  double src = -by_h(g, d, g.dx, g.rdx);
  d = sub(sub(add(y1[fy + g.nx], y2[fy + g.nx]), y1[fy]), y2[fy]);
  src = sub(src, by_h(g, d, g.dy, g.rdy));
  if (g.nz > 1) {
    const size_t pz = (size_t)g.nx * g.ny;
    d = sub(sub(add(z1[fz + pz], z2[fz + pz]), z1[fz]), z2[fz]);
    src = sub(src, by_h(g, d, g.dz, g.rdz));
  }
  double s;
  if (stage == 1) {
    l1[q] = src;
    s = src;
  } else if (stage == 2) {
    l2[q] = src;
    s = by4(add(mul(-3.0, l1[q]), src));
  } else {
    s = by12(add(sub(-l1[q], l2[q]), mul(8.0, src)));
  }
  phi[q] = add(phi[q], mul(s, dt));
}

// ---- redistancing: level_set_rk3_redis ("Two phase flows/newOpenMP/2D/src/
// interface_solver/level_set_rk3_redis.f90:1-361"; 3D "Two phase flows/
// newOpenMP/3D+IBM/src/interface_solver/level_set_rk3_redis.f90") ----------
constexpr double kPi = 3.141592653589793;  // acos(-1) in double

// ls_funs ("Two phase flows/newOpenMP/3D+IBM/src/interface_solver/
// others.f90:1-37"): smoothed Heaviside, its derivative and the sign 2H - 1
__device__ __forceinline__ void ls_funs1(double phi, double ls_wid, double& heavy, double& delta,
                                         double& sgn) {
  const double eps = 1.0e-12;
  const double x = dvd(phi, ls_wid);
  double h, hp;
  if (x > 1.0 - eps) {
    h = 1.0;
    hp = 0.0;
  } else if (x < -1.0 + eps) {
    h = 0.0;
    hp = 0.0;
  } else {
    h = mul(0.5, add(add(1.0, x), dvd(sin(mul(kPi, x)), kPi)));
    hp = dvd(mul(0.5, add(1.0, cos(mul(kPi, x)))), ls_wid);
  }
  h = h < 1.0 ? h : 1.0;
  h = h > 0.0 ? h : 0.0;
  heavy = h;
  delta = hp;
  sgn = sub(mul(2.0, h), 1.0);
}

// s = the sign held fixed through the call: 2H - 1, or phi itself for the
// first redistancing (level_set_redis_stable, btn = 0)
__global__ void __launch_bounds__(256) k_ls_sign(size_t n, const double* __restrict__ phi,
                                                 double ls_wid, int btn, double* __restrict__ s) {
  const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  if (btn == 0) {
    s[q] = phi[q];
  } else {
    double hv, dl, sg;
    ls_funs1(phi[q], ls_wid, hv, dl, sg);
    s[q] = sg;
  }
}

__device__ __forceinline__ double dmin(double a, double b) { return a < b ? a : b; }
__device__ __forceinline__ double dmax(double a, double b) { return a > b ? a : b; }

// |grad phi| by Godunov upwinding on the sign s (level_set_redis_gradient):
// the WENO-JS one-sided values (EPS = 1e-10) of the backward differences
// (phi_i - phi_{i-1})/h, zero-gradient ghosts by index clamping
__global__ void __launch_bounds__(256) k_ls_grad(LsGrid g, const double* __restrict__ phi,
                                                 const double* __restrict__ s,
                                                 double* __restrict__ grad) {
  const size_t n = (size_t)g.nx * g.ny * g.nz;
  const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const int i = (int)(q % g.nx);
  const size_t r = q / g.nx;
  const int j = (int)(r % g.ny), k = (int)(r / g.ny);
  const int naxes = g.nz > 1 ? 3 : 2;
  const bool pos = s[q] >= 0.0;
  double sum = 0.0;
  for (int a = 0; a < naxes; ++a) {
    const int n_a = a == 0 ? g.nx : (a == 1 ? g.ny : g.nz);
    const int c = a == 0 ? i : (a == 1 ? j : k);
    const size_t stride = a == 0 ? 1 : (a == 1 ? (size_t)g.nx : (size_t)g.nx * g.ny);
    const double h = a == 0 ? g.dx : (a == 1 ? g.dy : g.dz);
    const double rh = a == 0 ? g.rdx : (a == 1 ? g.rdy : g.rdz);
    const size_t base = q - (size_t)c * stride;
    double f[6];
#pragma unroll
    for (int m = 0; m < 6; ++m) {
      const int cc = clampi(c - 2 + m, n_a);
      const int cm = cc > 0 ? cc - 1 : 0;
      f[m] = by_h(g, sub(phi[base + (size_t)cc * stride], phi[base + (size_t)cm * stride]), h, rh);
    }
    const double s1 = weno_right(f[1], f[2], f[3], f[4], f[5], 1.0e-10);
    const double s2 = weno_left(f[0], f[1], f[2], f[3], f[4], 1.0e-10);
    const double pm = -dmin(s1, 0.0), pp = dmax(s1, 0.0);
    const double mm = -dmin(s2, 0.0), mp = dmax(s2, 0.0);
    const double t = pos ? dmax(pm, mp) : dmax(pp, mm);
    sum = a == 0 ? mul(t, t) : add(sum, mul(t, t));
  }
  grad[q] = __dsqrt_rn(sum);
}

// s2 = lam s (|grad| - 1), s3 = |grad| delta lam (level_set_redis_lambda)
__global__ void __launch_bounds__(256) k_ls_lambda(size_t n, int three, double ls_wid,
                                                   double rho12, const double* __restrict__ phi,
                                                   const double* __restrict__ s,
                                                   const double* __restrict__ grad,
                                                   double* __restrict__ s2,
                                                   double* __restrict__ s3) {
  const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  double hv, dl, sg;
  ls_funs1(phi[q], ls_wid, hv, dl, sg);
  const double lam = three ? mul(add(mul(mul(2.0, sub(1.0, rho12)), hv), rho12), dl) : dl;
  s2[q] = mul(mul(lam, s[q]), sub(grad[q], 1.0));
  s3[q] = mul(mul(grad[q], dl), lam);
}

// One pseudo-time stage: s1 = the correction (block sums of s2 and s3 with
// weight 16 (2D) or 51 (3D) on the cell, btn = 1; 0 for btn = 0),
// l = (s - s1)|grad| - s, phi -= rdt * (the stage's combination of l1..l3)
__global__ void __launch_bounds__(256) k_ls_redis_stage(LsGrid g, int stage, int btn, double rdt,
                                                        double ls_wid,
                                                        const double* __restrict__ s,
                                                        const double* __restrict__ grad,
                                                        const double* __restrict__ s2,
                                                        const double* __restrict__ s3,
                                                        double* l1, double* l2, double* phi) {
  const size_t n = (size_t)g.nx * g.ny * g.nz;
  const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  double s1 = 0.0;
  if (btn != 0) {
    const int i = (int)(q % g.nx);
    const size_t r = q / g.nx;
    const int j = (int)(r % g.ny), k = (int)(r / g.ny);
    const bool three = g.nz > 1;
    const double wgt = three ? 51.0 : 16.0;
    double a = mul(wgt, s2[q]), b = mul(wgt, s3[q]);
    const int k0 = three ? -1 : 0, k1 = three ? 1 : 0;
    for (int kk = k0; kk <= k1; ++kk)
      for (int jj = -1; jj <= 1; ++jj)
        for (int ii = -1; ii <= 1; ++ii) {
          const size_t rr = ((size_t)clampi(k + kk, g.nz) * g.ny + clampi(j + jj, g.ny)) * g.nx +
                            clampi(i + ii, g.nx);
          a = add(a, s2[rr]);
          b = add(b, s3[rr]);
        }
    double hv, dl, sg;
    ls_funs1(phi[q], ls_wid, hv, dl, sg);
    s1 = fabs(b) > 1.0e-12 ? mul(dvd(a, b), dl) : 0.0;
  }
  const double l = sub(mul(sub(s[q], s1), grad[q]), s[q]);
  double src;
  if (stage == 1) {
    l1[q] = l;
    src = l;
  } else if (stage == 2) {
    l2[q] = l;
    src = by4(add(mul(-3.0, l1[q]), l));
  } else {
    src = by12(add(sub(-l1[q], l2[q]), mul(8.0, l)));
  }
  phi[q] = sub(phi[q], mul(rdt, src));
}

// *out = max over cells of |a - b| (b == nullptr: max of a, a >= 0); the
// maximum of non-negative doubles is the maximum of their bit patterns
__global__ void __launch_bounds__(256) k_ls_maxabs(size_t n, const double* __restrict__ a,
                                                   const double* __restrict__ b,
                                                   unsigned long long* out) {
  double m = 0.0;
  for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < n;
       q += (size_t)gridDim.x * blockDim.x) {
    const double v = b ? fabs(sub(a[q], b[q])) : a[q];
    m = v > m ? v : m;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = dmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  __shared__ double ws[8];
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) m = dmax(m, ws[w]);
    atomicMax(out, (unsigned long long)__double_as_longlong(m));
  }
}

__global__ void k_ls_scale(size_t n, double* phi, const unsigned long long* gmax) {
  const double gm = __longlong_as_double((long long)*gmax);
  const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q < n) phi[q] = dvd(phi[q], gm);
}

inline unsigned blocks_for(size_t n) { return (unsigned)((n + 255) / 256); }

}  // namespace

}  // namespace gbmg

using namespace gbmg;

struct gbmg_ls {
  gbmg_grid grid{};
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  double *phi = nullptr, *u = nullptr, *v = nullptr, *w = nullptr, *l1 = nullptr, *l2 = nullptr;
  double* face[6] = {};
  unsigned long long* red = nullptr;  // one max-reduction slot
  unsigned long long* host_red = nullptr;
  int64_t launches = 0;
  std::string err;
};

namespace {

int ls_fail(gbmg_ls* ls, cudaError_t e, const char* what) {
  ls->err = std::string(what) + ": " + cudaGetErrorString(e);
  return e == cudaErrorMemoryAllocation ? GBMG_OUT_OF_MEMORY : GBMG_CUDA_ERROR;
}

#define LS_CUDA(ls, call)                              \
  do {                                                 \
    cudaError_t e_ = (call);                           \
    if (e_ != cudaSuccess) return ls_fail(ls, e_, #call); \
  } while (0)

size_t ls_cells(const gbmg_grid& g) { return (size_t)g.nx * g.ny * g.nz; }

void ls_free(gbmg_ls* ls) {
  double** all[] = {&ls->phi, &ls->u, &ls->v, &ls->w, &ls->l1, &ls->l2, &ls->face[0], &ls->face[1],
                    &ls->face[2], &ls->face[3], &ls->face[4], &ls->face[5]};
  for (double** p : all)
    if (*p) {
      cudaFree(*p);
      *p = nullptr;
    }
  if (ls->red) cudaFree(ls->red);
  if (ls->host_red) cudaFreeHost(ls->host_red);
  ls->red = nullptr;
  ls->host_red = nullptr;
}

// host or device field (strided, x contiguous) -> dense device array
int ls_in(gbmg_ls* ls, const gbmg_field& f, int mem, double* dst) {
  const gbmg_grid& g = ls->grid;
  if (!f.data || f.sy < g.nx || f.sz < f.sy * (int64_t)g.ny) {
    ls->err = "invalid field";
    return GBMG_INVALID_ARG;
  }
  const bool dense = f.sy == g.nx && f.sz == (int64_t)g.nx * g.ny;
  if (dense) {
    LS_CUDA(ls, cudaMemcpyAsync(dst, f.data, ls_cells(g) * sizeof(double),
                                mem == GBMG_MEM_HOST ? cudaMemcpyHostToDevice
                                                     : cudaMemcpyDeviceToDevice,
                                ls->stream));
  } else if (mem == GBMG_MEM_DEVICE) {
    launch_copy_in(ls->stream, g.nx, g.ny, g.nz, Strided{f.data, f.sy, f.sz}, dst);
    ls->launches += 1;
    LS_CUDA(ls, cudaGetLastError());
  } else {
    for (int k = 0; k < g.nz; ++k)
      LS_CUDA(ls, cudaMemcpy2DAsync(dst + (size_t)k * g.nx * g.ny, (size_t)g.nx * sizeof(double),
                                    f.data + (int64_t)k * f.sz, (size_t)f.sy * sizeof(double),
                                    (size_t)g.nx * sizeof(double), (size_t)g.ny,
                                    cudaMemcpyHostToDevice, ls->stream));
  }
  return GBMG_OK;
}

int ls_out(gbmg_ls* ls, const double* src, int mem, const gbmg_field& f) {
  const gbmg_grid& g = ls->grid;
  const bool dense = f.sy == g.nx && f.sz == (int64_t)g.nx * g.ny;
  if (dense) {
    LS_CUDA(ls, cudaMemcpyAsync(f.data, src, ls_cells(g) * sizeof(double),
                                mem == GBMG_MEM_HOST ? cudaMemcpyDeviceToHost
                                                     : cudaMemcpyDeviceToDevice,
                                ls->stream));
  } else if (mem == GBMG_MEM_DEVICE) {
    launch_copy_out(ls->stream, g.nx, g.ny, g.nz, src, f.data, f.sy, f.sz);
    ls->launches += 1;
    LS_CUDA(ls, cudaGetLastError());
  } else {
    for (int k = 0; k < g.nz; ++k)
      LS_CUDA(ls, cudaMemcpy2DAsync(f.data + (int64_t)k * f.sz, (size_t)f.sy * sizeof(double),
                                    src + (size_t)k * g.nx * g.ny, (size_t)g.nx * sizeof(double),
                                    (size_t)g.nx * sizeof(double), (size_t)g.ny,
                                    cudaMemcpyDeviceToHost, ls->stream));
  }
  return GBMG_OK;
}

}  // namespace

extern "C" {

int gbmg_ls_create(const gbmg_grid* grid, int device, void* stream, gbmg_ls** out) {
  if (!grid || !out) return GBMG_INVALID_ARG;
  *out = nullptr;
  if (grid->nx < 1 || grid->ny < 1 || grid->nz < 1 || !(grid->dx > 0) || !(grid->dy > 0) ||
      (grid->nz > 1 && !(grid->dz > 0)))
    return GBMG_INVALID_ARG;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) return GBMG_NO_DEVICE;
  gbmg_ls* ls = new gbmg_ls();
  ls->grid = *grid;
  if (device < 0) cudaGetDevice(&device);
  ls->device = device;
  if (cudaSetDevice(device) != cudaSuccess) {
    delete ls;
    return GBMG_NO_DEVICE;
  }
  if (stream) {
    ls->stream = static_cast<cudaStream_t>(stream);
  } else {
    if (cudaStreamCreateWithFlags(&ls->stream, cudaStreamNonBlocking) != cudaSuccess) {
      delete ls;
      return GBMG_CUDA_ERROR;
    }
    ls->own_stream = true;
  }
  const gbmg_grid& g = *grid;
  const size_t n = ls_cells(g);
  const size_t nfx = (size_t)(g.nx + 1) * g.ny * g.nz, nfy = (size_t)g.nx * (g.ny + 1) * g.nz,
               nfz = (size_t)g.nx * g.ny * (g.nz + 1);
  const size_t sizes[12] = {n, n, n, n, n, n, nfx, nfx, nfy, nfy, nfz, nfz};
  double** ptrs[12] = {&ls->phi, &ls->u, &ls->v, &ls->w, &ls->l1, &ls->l2, &ls->face[0],
                       &ls->face[1], &ls->face[2], &ls->face[3], &ls->face[4], &ls->face[5]};
  for (int a = 0; a < 12; ++a) {
    if (cudaMalloc((void**)ptrs[a], sizes[a] * sizeof(double)) != cudaSuccess) {
      cudaGetLastError();
      ls_free(ls);
      if (ls->own_stream) cudaStreamDestroy(ls->stream);
      delete ls;
      return GBMG_OUT_OF_MEMORY;
    }
  }
  if (cudaMalloc((void**)&ls->red, sizeof(unsigned long long)) != cudaSuccess ||
      cudaMallocHost((void**)&ls->host_red, sizeof(unsigned long long)) != cudaSuccess) {
    cudaGetLastError();
    ls_free(ls);
    if (ls->own_stream) cudaStreamDestroy(ls->stream);
    delete ls;
    return GBMG_OUT_OF_MEMORY;
  }
  *out = ls;
  return GBMG_OK;
}

int gbmg_ls_destroy(gbmg_ls* ls) {
  if (!ls) return GBMG_INVALID_ARG;
  cudaSetDevice(ls->device);
  if (ls->stream) cudaStreamSynchronize(ls->stream);
  ls_free(ls);
  if (ls->own_stream && ls->stream) cudaStreamDestroy(ls->stream);
  delete ls;
  return GBMG_OK;
}

int gbmg_ls_advect(gbmg_ls* ls, gbmg_field phi, gbmg_field u, gbmg_field v, gbmg_field w,
                   double dt, int steps, int mem) {
  if (!ls) return GBMG_INVALID_ARG;
  ls->err.clear();
  if (cudaSetDevice(ls->device) != cudaSuccess) {
    ls->err = "cudaSetDevice failed";
    return GBMG_CUDA_ERROR;
  }
  if (!(dt > 0) || steps < 0) {
    ls->err = "dt must be > 0 and steps >= 0";
    return GBMG_INVALID_ARG;
  }
  if (mem != GBMG_MEM_HOST && mem != GBMG_MEM_DEVICE) {
    ls->err = "mem must be GBMG_MEM_HOST or GBMG_MEM_DEVICE";
    return GBMG_INVALID_ARG;
  }
  const gbmg_grid& g = ls->grid;
  const bool three = g.nz > 1;
  int rc;
  if ((rc = ls_in(ls, phi, mem, ls->phi)) != GBMG_OK) return rc;
  if ((rc = ls_in(ls, u, mem, ls->u)) != GBMG_OK) return rc;
  if ((rc = ls_in(ls, v, mem, ls->v)) != GBMG_OK) return rc;
  if (three && (rc = ls_in(ls, w, mem, ls->w)) != GBMG_OK) return rc;
  const LsGrid G = ls_grid(g);
  const size_t n = ls_cells(g);
  const double* vel[3] = {ls->u, ls->v, ls->w};
  const size_t nf[3] = {(size_t)(g.nx + 1) * g.ny * g.nz, (size_t)g.nx * (g.ny + 1) * g.nz,
                        (size_t)g.nx * g.ny * (g.nz + 1)};
  for (int s = 0; s < steps; ++s)
    for (int stage = 1; stage <= 3; ++stage) {
      for (int a = 0; a < (three ? 3 : 2); ++a) {
        k_ls_faces<<<blocks_for(nf[a]), 256, 0, ls->stream>>>(G, a, ls->phi, vel[a],
                                                              ls->face[2 * a], ls->face[2 * a + 1]);
        ls->launches += 1;
      }
      k_ls_stage<<<blocks_for(n), 256, 0, ls->stream>>>(
          G, stage, dt, ls->face[0], ls->face[1], ls->face[2], ls->face[3], ls->face[4],
          ls->face[5], ls->l1, ls->l2, ls->phi);
      ls->launches += 1;
    }
  LS_CUDA(ls, cudaGetLastError());
  if ((rc = ls_out(ls, ls->phi, mem, phi)) != GBMG_OK) return rc;
  LS_CUDA(ls, cudaStreamSynchronize(ls->stream));
  return GBMG_OK;
}

namespace {
// max over cells of |a - b| (or of a), read back to the host
int ls_max(gbmg_ls* ls, const double* a, const double* b, double* out) {
  const size_t n = ls_cells(ls->grid);
  LS_CUDA(ls, cudaMemsetAsync(ls->red, 0, sizeof(unsigned long long), ls->stream));
  unsigned blocks = blocks_for(n);
  if (blocks > 1024) blocks = 1024;
  k_ls_maxabs<<<blocks, 256, 0, ls->stream>>>(n, a, b, ls->red);
  ls->launches += 1;
  LS_CUDA(ls, cudaGetLastError());
  LS_CUDA(ls, cudaMemcpyAsync(ls->host_red, ls->red, sizeof(unsigned long long),
                              cudaMemcpyDeviceToHost, ls->stream));
  LS_CUDA(ls, cudaStreamSynchronize(ls->stream));
  long long bits = (long long)*ls->host_red;
  std::memcpy(out, &bits, sizeof(double));
  return GBMG_OK;
}
}  // namespace

int gbmg_ls_redistance(gbmg_ls* ls, gbmg_field phi, double ls_wid, double rdt, double rho_12,
                       int btn, int max_iter, int mem, int32_t* iters, double* last_change) {
  if (!ls) return GBMG_INVALID_ARG;
  ls->err.clear();
  if (iters) *iters = 0;
  if (last_change) *last_change = 0.0;
  if (cudaSetDevice(ls->device) != cudaSuccess) {
    ls->err = "cudaSetDevice failed";
    return GBMG_CUDA_ERROR;
  }
  if (!(ls_wid > 0) || !(rdt > 0) || max_iter < 0 || (btn != 0 && btn != 1)) {
    ls->err = "ls_wid and rdt must be > 0, max_iter >= 0, btn 0 or 1";
    return GBMG_INVALID_ARG;
  }
  if (mem != GBMG_MEM_HOST && mem != GBMG_MEM_DEVICE) {
    ls->err = "mem must be GBMG_MEM_HOST or GBMG_MEM_DEVICE";
    return GBMG_INVALID_ARG;
  }
  const gbmg_grid& g = ls->grid;
  const bool three = g.nz > 1;
  const LsGrid G = ls_grid(g);
  const size_t n = ls_cells(g);
  const unsigned nb = blocks_for(n);
  double* s = ls->face[0];
  double* grad = ls->face[1];
  double* s2 = ls->face[2];
  double* s3 = ls->face[3];
  double* tmp = ls->face[4];
  int rc;
  if ((rc = ls_in(ls, phi, mem, ls->phi)) != GBMG_OK) return rc;
  // level_set_redis_init (+ level_set_redis_stable for btn = 0)
  k_ls_sign<<<nb, 256, 0, ls->stream>>>(n, ls->phi, ls_wid, btn, s);
  ls->launches += 1;
  if (btn == 0) {
    k_ls_grad<<<nb, 256, 0, ls->stream>>>(G, ls->phi, s, grad);
    ls->launches += 1;
    LS_CUDA(ls, cudaMemsetAsync(ls->red, 0, sizeof(unsigned long long), ls->stream));
    unsigned blocks = nb > 1024 ? 1024 : nb;
    k_ls_maxabs<<<blocks, 256, 0, ls->stream>>>(n, grad, nullptr, ls->red);
    k_ls_scale<<<nb, 256, 0, ls->stream>>>(n, ls->phi, ls->red);
    ls->launches += 2;
  }
  LS_CUDA(ls, cudaGetLastError());
  const double ext = three ? std::max(std::max(g.nx * g.dx, g.ny * g.dy), g.nz * g.dz)
                           : std::max(g.nx * g.dx, g.ny * g.dy);
  const double timestop = btn == 0 ? 1.5 * ext : 3.0 * g.dx;
  const double tol = three ? 1.0e-5 : 1.0e-8;
  double time = 0.0, error = 0.0;
  int iter = 0;
  while (iter < max_iter) {
    ++iter;
    time = time + rdt;
    LS_CUDA(ls, cudaMemcpyAsync(tmp, ls->phi, n * sizeof(double), cudaMemcpyDeviceToDevice,
                                ls->stream));
    for (int stage = 1; stage <= 3; ++stage) {
      k_ls_grad<<<nb, 256, 0, ls->stream>>>(G, ls->phi, s, grad);
      ls->launches += 1;
      if (btn != 0) {
        k_ls_lambda<<<nb, 256, 0, ls->stream>>>(n, three ? 1 : 0, ls_wid, rho_12, ls->phi, s,
                                                grad, s2, s3);
        ls->launches += 1;
      }
      k_ls_redis_stage<<<nb, 256, 0, ls->stream>>>(G, stage, btn, rdt, ls_wid, s, grad, s2, s3,
                                                   ls->l1, ls->l2, ls->phi);
      ls->launches += 1;
    }
    LS_CUDA(ls, cudaGetLastError());
    if ((rc = ls_max(ls, tmp, ls->phi, &error)) != GBMG_OK) return rc;
    if (time > timestop || error <= tol) break;
  }
  if ((rc = ls_out(ls, ls->phi, mem, phi)) != GBMG_OK) return rc;
  LS_CUDA(ls, cudaStreamSynchronize(ls->stream));
  if (iters) *iters = iter;
  if (last_change) *last_change = error;
  return GBMG_OK;
}

int64_t gbmg_ls_kernel_launches(gbmg_ls* ls) { return ls ? ls->launches : 0; }

const char* gbmg_ls_last_error(gbmg_ls* ls) { return ls ? ls->err.c_str() : ""; }

}  // extern "C"
