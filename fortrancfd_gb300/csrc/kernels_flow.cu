// Projection-step kernels for sm_103a: level set -> density, density -> face
// coefficients, MAC divergence, pressure-gradient correction, divergence
// statistics, and the FP64 vector kernels of the solve loop (mean projection,
// mixed-precision update, flexible-CG steps).
//
// Reference loops: rho_mu / ls_funs ("Two phase flows/newOpenMP/2D/src/
// interface_solver/others.f90:1-61"), ppe_sor_init and ppe_sor_solver's RHS
// ("Two phase flows/newOpenMP/3D+IBM/src/ns_solver/ns_ppe_solver.f90:1-65,
// 77-89"), ns_momentum_correction (same file :174-205) and
// ns_check_convergence_div ("Two phase flows/newOpenMP/2D/src/ns_solver/
// ns_solvers.f90:55-83").
#include <algorithm>
#include <cmath>
#include <cstring>

#include "dword.cuh"
#include "gbmg_internal.h"
#include "reduce.cuh"

namespace gbmg {

namespace {

inline unsigned cdiv(size_t a, unsigned b) { return (unsigned)((a + b - 1) / b); }

inline unsigned stride_blocks(size_t n) {
  const size_t b = cdiv(n, kRedThreads);
  return (unsigned)std::max<size_t>(1, std::min<size_t>(b, 152 * 8));
}

// Smoothed Heaviside H(phi/eps) = (1 + x + sin(pi x)/pi)/2 on |x| < 1, then
// rho = rho_pos H + rho_neg (1 - H).
// Outside the band |phi| > eps_out (eps_out slightly above eps (1 - 1e-12),
// set by the host) the division phi/eps would land past the clipping
// threshold anyway, so H is 0 or 1 without computing it: the same result as
// the full branch, with the FP64 division done only in the band.
// The outside test compares bit patterns (|phi| > eps_out as integers;
// NaN stays on the full branch), and outside cells store the two bulk values
// rho_pos*1 + rho_neg*0 and rho_pos*0 + rho_neg*1 computed by the host: the
// full formula's result for H = 1 and 0, without FP64 work.
constexpr int kRhoPlanes = 4;

__global__ void __launch_bounds__(256) k_rho_from_phi(int nx, int ny, int nz, Strided phi,
                                                      double eps, long long eps_out_bits,
                                                      double rho_pos, double rho_neg,
                                                      double bulk_pos, double bulk_neg,
                                                      double* rho) {
  // four z planes per thread, their loads issued together
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k0 = blockIdx.z * kRhoPlanes;
  if (i >= nx || j >= ny) return;
  const double pi = 3.141592653589793;
  double ph[kRhoPlanes];
#pragma unroll
  for (int u = 0; u < kRhoPlanes; ++u)
    ph[u] = k0 + u < nz ? phi.data[i + j * phi.sy + (int64_t)(k0 + u) * phi.sz] : 0.0;
#pragma unroll
  for (int u = 0; u < kRhoPlanes; ++u) {
    const int k = k0 + u;
    if (k >= nz) break;
    const long long pb = __double_as_longlong(ph[u]);
    const long long mag = pb & 0x7fffffffffffffffll;
    double* out = rho + ((size_t)k * ny + j) * nx + i;
    if (mag > eps_out_bits && mag <= 0x7ff0000000000000ll) {
      *out = pb < 0 ? bulk_neg : bulk_pos;
      continue;
    }
    double h;
    const double x = ph[u] / eps;
    if (x > 1.0 - 1e-12) h = 1.0;
    else if (x < -1.0 + 1e-12) h = 0.0;
    else h = 0.5 * (1.0 + x + sin(pi * x) / pi);
    h = fmax(fmin(h, 1.0), 0.0);
    *out = rho_pos * h + rho_neg * (1.0 - h);
  }
}

__global__ void __launch_bounds__(256) k_copy_in(int nx, int ny, int nz, Strided src, double* dst) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i >= nx || j >= ny) return;
  dst[((size_t)k * ny + j) * nx + i] = src.data[i + j * src.sy + k * src.sz];
}

__global__ void __launch_bounds__(256) k_copy_out(int nx, int ny, int nz, const double* src,
                                                  double* dst, int64_t sy, int64_t sz) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i >= nx || j >= ny) return;
  dst[i + j * sy + k * sz] = src[((size_t)k * ny + j) * nx + i];
}

// coe = 2/(rho_i + rho_nb)/h^2 on the low face of every cell, 0 on the walls
// (the reference's arithmetic, ns_ppe_solver.f90:12-24, so the operator is
// bit-identical to the oracle's).  When h^2 is a power of two the division by
// it is an exact scaling and is done as a multiplication by 1/h^2 (same
// result, one FP64 division instead of two).  Optionally also writes the
// FP32 copies of the cycle and the double-word copies of the defect kernel.
struct BulkFaces {
  long long r[2];     // bit patterns of the two bulk densities (never equal to a double
                      // when there are none: a NaN pattern no density takes)
  double c[3][2];     // face coefficient per axis and bulk density
  float c32[3][2];
  float2 cw[3][2];
};

struct FaceOut {
  double* c;
  float* c32;
  float2* cw;
};

__device__ __forceinline__ void face_store(const FaceOut& o, size_t q, double v) {
  o.c[q] = v;
  if (o.c32) o.c32[q] = (float)v;
  if (o.cw) {
    const dw d = dw_from_double_int(v);
    o.cw[q] = make_float2(d.hi, d.lo);
  }
}

// The face value for rho_i + rho_nb = s along axis a (0 on walls); faces
// between two cells of a bulk density (s equal to one of the two precomputed
// sums) take the host-computed values, computed with the same IEEE operations.
// ra, rb: the two cells' densities.  The bulk test compares bit patterns
// (integer operations; FP64 compares and adds run at GB300's FP64 rate).
__device__ __forceinline__ void face_value(const BulkFaces& B, int a, double ra, double rb,
                                           double h2, double ih2, bool pow2, const FaceOut& o,
                                           size_t q) {
  const long long ba = __double_as_longlong(ra), bb = __double_as_longlong(rb);
  for (int v = 0; v < 2; ++v)
    if (ba == B.r[v] && bb == B.r[v]) {
      o.c[q] = B.c[a][v];
      if (o.c32) o.c32[q] = B.c32[a][v];
      if (o.cw) o.cw[q] = B.cw[a][v];
      return;
    }
  const double t = 2.0 / (ra + rb);
  face_store(o, q, pow2 ? t * ih2 : t / h2);
}

__global__ void __launch_bounds__(256) k_face_coef(int nx, int ny, int nz, double3 h2, double3 ih2,
                                                   int pow2, BulkFaces B,
                                                   const double* __restrict__ rho, FaceOut ox,
                                                   FaceOut oy, FaceOut oz, float* rho32,
                                                   size_t hstride) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i >= nx || j >= ny) return;
  const size_t q = ((size_t)k * ny + j) * nx + i;
  const double r = rho[q];
  // the FP32 density of the mixed cycle (rounded to nearest; colour-split
  // when hstride != 0)
  if (rho32) rho32[hstride ? (size_t)((i + j + k) & 1) * hstride + (q >> 1) : q] =
      dw_from_double_int(r).hi;
  if (i > 0) face_value(B, 0, r, rho[q - 1], h2.x, ih2.x, pow2 & 1, ox, q);
  else face_store(ox, q, 0.0);
  if (j > 0) face_value(B, 1, r, rho[q - nx], h2.y, ih2.y, pow2 & 2, oy, q);
  else face_store(oy, q, 0.0);
  if (k > 0) face_value(B, 2, r, rho[q - (size_t)nx * ny], h2.z, ih2.z, pow2 & 4, oz, q);
  else face_store(oz, q, 0.0);
}

// b = div(u)/dt with MAC faces: u(f,j,k) on the x-face at f*dx, f = 0..nx.
// x / h, as a product with the exact reciprocal when h is a power of two
// (bit-identical to the division and without its FP64 cost); pow2 is the
// host's is_pow2(h), ih = 1/h.
__device__ __forceinline__ double over(double x, double h, double ih, bool pow2) {
  return pow2 ? x * ih : x / h;
}

__global__ void __launch_bounds__(256) k_divergence(int nx, int ny, int nz, Strided u, Strided v,
                                                    Strided w, double3 h, double3 ih, int pow2,
                                                    double dt, double* b) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i >= nx || j >= ny) return;
  const int64_t qu = i + j * u.sy + k * u.sz;
  const int64_t qv = i + j * v.sy + k * v.sz;
  double d = over(u.data[qu + 1] - u.data[qu], h.x, ih.x, pow2 & 1) +
             over(v.data[qv + v.sy] - v.data[qv], h.y, ih.y, pow2 & 2);
  if (w.data) {
    const int64_t qw = i + j * w.sy + k * w.sz;
    d += over(w.data[qw + w.sz] - w.data[qw], h.z, ih.z, pow2 & 4);
  }
  b[((size_t)k * ny + j) * nx + i] = d / dt;
}

// u_f -= dt (p_i - p_{i-1})/dx / ((rho_i + rho_{i-1})/2) on every interior
// face; each cell corrects its low faces.
// (halving is exact, so /2 is taken as *0.5)
__global__ void __launch_bounds__(256) k_correct(int nx, int ny, int nz,
                                                 const double* __restrict__ rho,
                                                 const double* __restrict__ p, double3 h,
                                                 double3 ih, int pow2, double dt, double* u,
                                                 int64_t usy, int64_t usz, double* v, int64_t vsy,
                                                 int64_t vsz, double* w, int64_t wsy, int64_t wsz) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i >= nx || j >= ny) return;
  const size_t q = ((size_t)k * ny + j) * nx + i;
  if (i > 0) {
    const double rf = (rho[q] + rho[q - 1]) * 0.5;
    const double px = over(p[q] - p[q - 1], h.x, ih.x, pow2 & 1);
    u[i + j * usy + k * usz] -= dt * px / rf;
  }
  if (j > 0) {
    const double rf = (rho[q] + rho[q - nx]) * 0.5;
    const double py = over(p[q] - p[q - nx], h.y, ih.y, pow2 & 2);
    v[i + j * vsy + k * vsz] -= dt * py / rf;
  }
  if (k > 0 && w) {
    const size_t sz = (size_t)nx * ny;
    const double rf = (rho[q] + rho[q - sz]) * 0.5;
    const double pz = over(p[q] - p[q - sz], h.z, ih.z, pow2 & 4);
    w[i + j * wsy + k * wsz] -= dt * pz / rf;
  }
}

// Adjoint of the solve with respect to the density (and the level set):
// dJ/drho_i = sum over the faces of cell i of (lam_nb - lam_i)(p_nb - p_i)
// * (-2/(rho_i + rho_nb)^2/h^2); with phi, dJ/dphi = dJ/drho (rho_pos -
// rho_neg) H'(phi), H' = (1 + cos(pi phi/eps))/(2 eps) inside the band.
__global__ void __launch_bounds__(256) k_adjoint(int nx, int ny, int nz, double3 h2,
                                                 const double* __restrict__ rho,
                                                 const double* __restrict__ p,
                                                 const double* __restrict__ lam, Strided phi,
                                                 double eps, double rpos, double rneg,
                                                 double* grad_rho, double* grad_phi) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i >= nx || j >= ny) return;
  const size_t sy = (size_t)nx, sz = (size_t)nx * ny;
  const size_t q = (size_t)k * sz + (size_t)j * sy + i;
  const bool has[6] = {i > 0, i < nx - 1, j > 0, j < ny - 1, k > 0, k < nz - 1};
  const long long off[6] = {-1, 1, -(long long)sy, (long long)sy, -(long long)sz, (long long)sz};
  const double hh[3] = {h2.x, h2.y, h2.z};
  double acc = 0.0;
#pragma unroll
  for (int f = 0; f < 6; ++f) {
    if (!has[f]) continue;
    const size_t n = (size_t)((long long)q + off[f]);
    const double s = rho[q] + rho[n];
    const double dcoe = -2.0 / (s * s) / hh[f / 2];
    acc += (lam[n] - lam[q]) * (p[n] - p[q]) * dcoe;
  }
  grad_rho[q] = acc;
  if (grad_phi) {
    const double pi = 3.141592653589793;
    const double x = phi.data[i + j * phi.sy + k * phi.sz] / eps;
    const double hp =
        (x > 1.0 - 1e-12 || x < -1.0 + 1e-12) ? 0.0 : 0.5 * (1.0 + cos(pi * x)) / eps;
    grad_phi[q] = acc * (rpos - rneg) * hp;
  }
}

// max |div u| by atomicMax on the bit pattern (non-negative doubles order as
// unsigned integers) and sum |div u| through the deterministic reducer.
__global__ void __launch_bounds__(kRedThreads) k_div_stats(int nx, int ny, int nz, Strided u,
                                                           Strided v, Strided w, double dx,
                                                           double dy, double dz,
                                                           ReduceScratch R) {
  double acc[1] = {0.0};
  double mx = 0.0;
  const int rows = ny * nz;
  for (int row = blockIdx.x; row < rows; row += gridDim.x) {
    const int j = row % ny, k = row / ny;
    for (int i = threadIdx.x; i < nx; i += blockDim.x) {
      const int64_t qu = i + j * u.sy + k * u.sz;
      const int64_t qv = i + j * v.sy + k * v.sz;
      double d = (u.data[qu + 1] - u.data[qu]) / dx + (v.data[qv + v.sy] - v.data[qv]) / dy;
      if (w.data) {
        const int64_t qw = i + j * w.sy + k * w.sz;
        d += (w.data[qw + w.sz] - w.data[qw]) / dz;
      }
      d = fabs(d);
      mx = fmax(mx, d);
      acc[0] += d;
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_down_sync(0xffffffffu, mx, o));
  if ((threadIdx.x & 31) == 0)
    atomicMax(reinterpret_cast<unsigned long long*>(R.result + kSlotMax),
              (unsigned long long)__double_as_longlong(mx));
  grid_sum_finish<1>(acc, R, kSlotSum);
}

// The increment of one cycle for GBMG_STOP_INCREMENT: d = x - y (y may be
// null) over the cells (colour-split when hstride > 0: cells [0, n/2) of each
// half, the pad between the halves skipped).  The reference removes the mean
// of p before it measures the change (ppe_sor_solver, PRESS_POISSON), so the
// increment is max |d - mean(d)|: k_delta_sum sums d, k_delta_absmax takes
// the maximum of |d - mean| as a bit pattern (non-negative doubles order as
// unsigned integers) by atomicMax into R.result[slot_out].
template <typename T>
__device__ __forceinline__ size_t cell_index(size_t i, size_t n, size_t hstride) {
  return hstride ? (i < n / 2 ? i : hstride + (i - n / 2)) : i;
}

template <typename T>
__global__ void __launch_bounds__(kRedThreads) k_delta_sum(const T* __restrict__ x,
                                                           const T* __restrict__ y, size_t n,
                                                           size_t hstride, ReduceScratch R,
                                                           int slot) {
  double acc[1] = {0.0};
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const size_t q = cell_index<T>(i, n, hstride);
    acc[0] += y ? (double)x[q] - (double)y[q] : (double)x[q];
  }
  grid_sum_finish<1>(acc, R, slot);
}

template <typename T>
__global__ void __launch_bounds__(kRedThreads) k_delta_absmax(const T* __restrict__ x,
                                                              const T* __restrict__ y, size_t n,
                                                              size_t hstride, ReduceScratch R,
                                                              int slot_sum, int slot_out) {
  const double m = R.result[slot_sum] / (double)n;
  double mx = 0.0;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const size_t q = cell_index<T>(i, n, hstride);
    const double d = y ? (double)x[q] - (double)y[q] : (double)x[q];
    mx = fmax(mx, fabs(d - m));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_down_sync(0xffffffffu, mx, o));
  if ((threadIdx.x & 31) == 0)
    atomicMax(reinterpret_cast<unsigned long long*>(R.result + slot_out),
              (unsigned long long)__double_as_longlong(mx));
}

// RHSP's wall-normal faces set to zero: u at f = 0 and nx, v at 0 and ny, w at
// 0 and nz (arrays at face (0,0,0)); one thread per face of each wall pair.
__global__ void k_zero_wall_faces(int nx, int ny, int nz, double* u, int64_t usy, int64_t usz,
                                  double* v, int64_t vsy, int64_t vsz, double* w, int64_t wsy,
                                  int64_t wsz) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t nu = (int64_t)ny * nz, nv = (int64_t)nx * nz, nw = w ? (int64_t)nx * ny : 0;
  if (t < nu) {
    const int j = (int)(t % ny), k = (int)(t / ny);
    const int64_t q = j * usy + k * usz;
    u[q] = 0.0;
    u[q + nx] = 0.0;
  } else if (t < nu + nv) {
    const int64_t r = t - nu;
    const int i = (int)(r % nx), k = (int)(r / nx);
    const int64_t q = i + k * vsz;
    v[q] = 0.0;
    v[q + (int64_t)ny * vsy] = 0.0;
  } else if (t < nu + nv + nw) {
    const int64_t r = t - nu - nv;
    const int i = (int)(r % nx), j = (int)(r / nx);
    const int64_t q = i + j * wsy;
    w[q] = 0.0;
    w[q + (int64_t)nz * wsz] = 0.0;
  }
}

__global__ void __launch_bounds__(kRedThreads) k_sum(const double* __restrict__ x, size_t n,
                                                     ReduceScratch R, int slot) {
  double acc[2] = {0.0, 0.0};
  stride4(n, [&](size_t q) { return x[q]; }, [&](size_t, double a) {
    acc[0] += a;
    acc[1] += a * a;
  });
  grid_sum_finish<2>(acc, R, slot);
}

__global__ void __launch_bounds__(kRedThreads) k_shift_by_mean(const double* __restrict__ x,
                                                               double* y, size_t n,
                                                               ReduceScratch R, int slot,
                                                               int slot2) {
  const double m = R.result[slot] / (double)n;
  double acc[1] = {0.0};
  stride4(n, [&](size_t q) { return x[q]; }, [&](size_t q, double xq) {
    const double a = xq - m;
    y[q] = a;
    acc[0] += a * a;
  });
  if (slot2 >= 0) grid_sum_finish<1>(acc, R, slot2);
}

__global__ void k_add_float(double* p, const float* __restrict__ e, size_t n) {
  stride4(n, [&](size_t q) { return make_double2(p[q], (double)e[q]); },
          [&](size_t q, double2 v) { p[q] = v.x + v.y; });
}

__global__ void k_f2d(const float* __restrict__ a, double* b, size_t n) {
  stride4(n, [&](size_t q) { return a[q]; }, [&](size_t q, float v) { b[q] = (double)v; });
}

__global__ void k_d2f(const double* __restrict__ a, float* b, size_t n) {
  stride4(n, [&](size_t q) { return a[q]; }, [&](size_t q, double v) { b[q] = (float)v; });
}

// slot <- a.b, slot+1 <- a.c (c may be null)
__global__ void __launch_bounds__(kRedThreads) k_dot2(const double* __restrict__ a,
                                                      const double* __restrict__ b,
                                                      const double* __restrict__ c, size_t n,
                                                      ReduceScratch R, int slot) {
  double acc[2] = {0.0, 0.0};
  stride4(n, [&](size_t q) { return make_double3(a[q], b[q], c ? c[q] : 0.0); },
          [&](size_t, double3 v) {
            acc[0] += v.x * v.y;
            if (c) acc[1] += v.x * v.z;
          });
  grid_sum_finish<2>(acc, R, slot);
}

// Flexible-CG direction: beta = (r.z - r.z_old)/rz_old (0 on the first
// iteration), d = z + beta d, z_old = z.  rz_old lives in result[kSlotDot2+1].
__global__ void k_pcg_direction(double* d, double* zold, const double* __restrict__ z, size_t n,
                                ReduceScratch R, int first) {
  const double rz = R.result[kSlotDot], rzo = R.result[kSlotDot + 1];
  const double beta = first ? 0.0 : (rz - rzo) / R.result[kSlotDot2 + 1];
  stride4(n, [&](size_t q) { return make_double2(z[q], first ? 0.0 : d[q]); },
          [&](size_t q, double2 v) {
            d[q] = first ? v.x : v.x + beta * v.y;
            zold[q] = v.x;
          });
}

__global__ void k_pcg_keep_rz(ReduceScratch R) { R.result[kSlotDot2 + 1] = R.result[kSlotDot]; }

// x += alpha d with alpha = (r.z)/(d.q)
__global__ void k_pcg_step(double* x, const double* __restrict__ d, size_t n, ReduceScratch R) {
  const double alpha = R.result[kSlotDot] / R.result[kSlotDot2];
  stride4(n, [&](size_t q) { return make_double2(x[q], d[q]); },
          [&](size_t q, double2 v) { x[q] = v.x + alpha * v.y; });
}

}  // namespace

// ---------------------------------------------------------------------------
static inline dim3 grid3(int nx, int ny, int nz) {
  return dim3(cdiv((size_t)nx, 32), cdiv((size_t)ny, 8), (unsigned)nz);
}

void launch_rho_from_phi(cudaStream_t s, int nx, int ny, int nz, Strided phi, double eps,
                         double rho_pos, double rho_neg, double* rho) {
  // |phi| > eps_out implies |fl(phi/eps)| > 1 - 1e-12 (margin 1e-15 >> rounding)
  const double eps_out = eps * (1.0 - 1e-12) * (1.0 + 1e-15);
  long long eps_bits;
  std::memcpy(&eps_bits, &eps_out, sizeof eps_bits);
  const double bulk_pos = rho_pos * 1.0 + rho_neg * (1.0 - 1.0);
  const double bulk_neg = rho_pos * 0.0 + rho_neg * (1.0 - 0.0);
  const dim3 g(cdiv((size_t)nx, 32), cdiv((size_t)ny, 8), cdiv((size_t)nz, kRhoPlanes));
  k_rho_from_phi<<<g, dim3(32, 8), 0, s>>>(
      nx, ny, nz, phi, eps, eps_bits, rho_pos, rho_neg, bulk_pos, bulk_neg, rho);
}

void launch_copy_in(cudaStream_t s, int nx, int ny, int nz, Strided src, double* dst) {
  k_copy_in<<<grid3(nx, ny, nz), dim3(32, 8), 0, s>>>(nx, ny, nz, src, dst);
}

void launch_copy_out(cudaStream_t s, int nx, int ny, int nz, const double* src, double* dst,
                     int64_t sy, int64_t sz) {
  k_copy_out<<<grid3(nx, ny, nz), dim3(32, 8), 0, s>>>(nx, ny, nz, src, dst, sy, sz);
}

static bool is_pow2(double v) {
  int e;
  return v > 0.0 && std::frexp(v, &e) == 0.5;
}

void launch_face_coef(cudaStream_t s, int nx, int ny, int nz, double dx2, double dy2, double dz2,
                      const double* rho, double* cx, double* cy, double* cz, float* const* c32,
                      float2* const* cw, const double* bulk_rho, float* rho32, size_t hstride) {
  const int pow2 = (is_pow2(dx2) ? 1 : 0) | (is_pow2(dy2) ? 2 : 0) | (is_pow2(dz2) ? 4 : 0);
  const double h2[3] = {dx2, dy2, dz2};
  BulkFaces B;
  for (int v = 0; v < 2; ++v) {
    double rv = std::nan("");
    if (bulk_rho) rv = bulk_rho[v];
    std::memcpy(&B.r[v], &rv, sizeof rv);
    if (!bulk_rho) B.r[v] = 0x7ff8dead0000beefll;  // a NaN pattern: matches no density
    const double sv = rv + rv;
    for (int a = 0; a < 3; ++a) {
      const double t = 2.0 / sv;
      const double c = ((pow2 >> a) & 1) ? t * (1.0 / h2[a]) : t / h2[a];
      B.c[a][v] = c;
      B.c32[a][v] = (float)c;
      const float hi = (float)c;
      B.cw[a][v] = make_float2(hi, (float)(c - (double)hi));
    }
  }
  const FaceOut ox{cx, c32 ? c32[0] : nullptr, cw ? cw[0] : nullptr};
  const FaceOut oy{cy, c32 ? c32[1] : nullptr, cw ? cw[1] : nullptr};
  const FaceOut oz{cz, c32 ? c32[2] : nullptr, cw ? cw[2] : nullptr};
  k_face_coef<<<grid3(nx, ny, nz), dim3(32, 8), 0, s>>>(
      nx, ny, nz, make_double3(dx2, dy2, dz2), make_double3(1.0 / dx2, 1.0 / dy2, 1.0 / dz2), pow2,
      B, rho, ox, oy, oz, rho32, hstride);
}

void launch_divergence(cudaStream_t s, int nx, int ny, int nz, Strided u, Strided v, Strided w,
                       double dx, double dy, double dz, double dt, double* b) {
  const int pow2 = (is_pow2(dx) ? 1 : 0) | (is_pow2(dy) ? 2 : 0) | (is_pow2(dz) ? 4 : 0);
  k_divergence<<<grid3(nx, ny, nz), dim3(32, 8), 0, s>>>(
      nx, ny, nz, u, v, w, make_double3(dx, dy, dz), make_double3(1.0 / dx, 1.0 / dy, 1.0 / dz),
      pow2, dt, b);
}

void launch_correct(cudaStream_t s, int nx, int ny, int nz, const double* rho, const double* p,
                    double dx, double dy, double dz, double dt, double* u, int64_t usy,
                    int64_t usz, double* v, int64_t vsy, int64_t vsz, double* w, int64_t wsy,
                    int64_t wsz) {
  const int pow2 = (is_pow2(dx) ? 1 : 0) | (is_pow2(dy) ? 2 : 0) | (is_pow2(dz) ? 4 : 0);
  k_correct<<<grid3(nx, ny, nz), dim3(32, 8), 0, s>>>(
      nx, ny, nz, rho, p, make_double3(dx, dy, dz), make_double3(1.0 / dx, 1.0 / dy, 1.0 / dz),
      pow2, dt, u, usy, usz, v, vsy, vsz, w, wsy, wsz);
}

void launch_adjoint(cudaStream_t s, int nx, int ny, int nz, double dx2, double dy2, double dz2,
                    const double* rho, const double* p, const double* lam, Strided phi,
                    double eps, double rpos, double rneg, double* grad_rho, double* grad_phi) {
  k_adjoint<<<grid3(nx, ny, nz), dim3(32, 8), 0, s>>>(nx, ny, nz, make_double3(dx2, dy2, dz2), rho,
                                                     p, lam, phi, eps, rpos, rneg, grad_rho,
                                                     grad_phi);
}

void launch_div_stats(cudaStream_t s, int nx, int ny, int nz, Strided u, Strided v, Strided w,
                      double dx, double dy, double dz, const ReduceScratch& R) {
  cudaMemsetAsync(R.result + kSlotMax, 0, sizeof(double), s);
  const int blocks = std::min(reduce_blocks_for((size_t)ny * nz), R.max_blocks);
  k_div_stats<<<blocks, kRedThreads, 0, s>>>(nx, ny, nz, u, v, w, dx, dy, dz, R);
}

// *flag |= 1 when any x[q] is nonzero (-0 counts as zero): bit tests only,
// so the pass runs at the memory rate whatever the FP64 rate
__global__ void __launch_bounds__(kRedThreads) k_nonzero(const double* __restrict__ x, size_t n,
                                                         unsigned long long* flag) {
  unsigned long long acc = 0ull;
  stride4(n, [&](size_t q) { return (unsigned long long)__double_as_longlong(x[q]); },
          [&](size_t, unsigned long long b) { acc |= b << 1; });
  if (__any_sync(0xffffffffu, acc != 0ull) && (threadIdx.x & 31) == 0) atomicOr(flag, 1ull);
}

__global__ void k_cycle_ctl(CycleCtl* c, const double* __restrict__ result,
                            cudaGraphConditionalHandle loop, cudaGraphConditionalHandle next,
                            int has_next) {
  c->cyc += c->step;
  c->iters += 1;
  const double prev = c->rel;
  const double r2 = result[kSlotNorm];
  const double rel = sqrt(r2) / c->scale;
  c->r2 = r2;
  c->rel = rel;
  int stop = 0;
  if (!isfinite(rel) || rel > c->guard) {
    c->status = kCtlDiverged;
    stop = 1;
  } else if (c->by_inc) {
    const double dp = result[kSlotInc];  // a non-negative double kept as its bit pattern
    c->inc = dp;
    if (dp < c->tol) {
      c->status = kCtlConverged;
      stop = 1;
    }
  } else if (rel < c->tol) {
    c->status = kCtlConverged;
    stop = 1;
  } else if (c->flat_stop) {
    if (rel < c->best) {
      c->best = rel;
      c->flat = 0;
    } else if (++c->flat >= 4) {
      c->stalled = 1;
      stop = 1;
    }
  }
  // stop before an iteration would pass the cycle limit (the host runs the
  // remaining cycles one at a time)
  if (!stop && c->adaptive) {
    const int k = tail_cycles(rel, prev, c->tol, c->step, c->step);
    if (k < c->step) {
      c->tail = k;
      stop = 1;
    }
  }
  if (!stop && c->cyc + c->step > c->max_cycles) stop = 1;
  cudaGraphSetConditional(loop, stop ? 0u : 1u);
  if (has_next) cudaGraphSetConditional(next, stop ? 0u : 1u);
}

void launch_cycle_ctl(cudaStream_t s, CycleCtl* c, const double* result,
                      cudaGraphConditionalHandle loop, cudaGraphConditionalHandle next,
                      int has_next) {
  k_cycle_ctl<<<1, 1, 0, s>>>(c, result, loop, next, has_next);
}

template <typename T>
void launch_increment(cudaStream_t s, const T* x, const T* y, size_t n, size_t hstride,
                      const ReduceScratch& R, int slot_sum, int slot_out) {
  const unsigned b = std::min<unsigned>(stride_blocks(n), (unsigned)R.max_blocks);
  k_delta_sum<T><<<b, kRedThreads, 0, s>>>(x, y, n, hstride, R, slot_sum);
  cudaMemsetAsync(R.result + slot_out, 0, sizeof(double), s);
  k_delta_absmax<T><<<stride_blocks(n), kRedThreads, 0, s>>>(x, y, n, hstride, R, slot_sum,
                                                             slot_out);
}
template void launch_increment<float>(cudaStream_t, const float*, const float*, size_t, size_t,
                                      const ReduceScratch&, int, int);
template void launch_increment<double>(cudaStream_t, const double*, const double*, size_t,
                                       size_t, const ReduceScratch&, int, int);

void launch_zero_wall_faces(cudaStream_t s, int nx, int ny, int nz, double* u, int64_t usy,
                            int64_t usz, double* v, int64_t vsy, int64_t vsz, double* w,
                            int64_t wsy, int64_t wsz) {
  const int64_t total = (int64_t)ny * nz + (int64_t)nx * nz + (w ? (int64_t)nx * ny : 0);
  k_zero_wall_faces<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(nx, ny, nz, u, usy, usz, v,
                                                                   vsy, vsz, w, wsy, wsz);
}

void launch_nonzero(cudaStream_t s, const double* x, size_t n, double* flag) {
  cudaMemsetAsync(flag, 0, sizeof(double), s);
  k_nonzero<<<stride_blocks(n) * 2, kRedThreads, 0, s>>>(
      x, n, reinterpret_cast<unsigned long long*>(flag));
}

void launch_sum(cudaStream_t s, const double* x, size_t n, const ReduceScratch& R, int slot) {
  const unsigned b = std::min<unsigned>(stride_blocks(n), (unsigned)R.max_blocks);
  k_sum<<<b, kRedThreads, 0, s>>>(x, n, R, slot);
}

void launch_shift_by_mean(cudaStream_t s, const double* x, double* y, size_t n,
                          const ReduceScratch& R, int slot, int slot2) {
  const unsigned b = std::min<unsigned>(stride_blocks(n), (unsigned)R.max_blocks);
  k_shift_by_mean<<<b, kRedThreads, 0, s>>>(x, y, n, R, slot, slot2);
}

void launch_add_float(cudaStream_t s, double* p, const float* e, size_t n) {
  k_add_float<<<stride_blocks(n) * 2, kRedThreads, 0, s>>>(p, e, n);
}

void launch_float_to_double(cudaStream_t s, const float* a, double* b, size_t n) {
  k_f2d<<<stride_blocks(n) * 2, kRedThreads, 0, s>>>(a, b, n);
}

void launch_double_to_float(cudaStream_t s, const double* a, float* b, size_t n) {
  k_d2f<<<stride_blocks(n) * 2, kRedThreads, 0, s>>>(a, b, n);
}

void launch_dot2(cudaStream_t s, const double* a, const double* b, const double* c, size_t n,
                 const ReduceScratch& R, int slot) {
  const unsigned bl = std::min<unsigned>(stride_blocks(n), (unsigned)R.max_blocks);
  k_dot2<<<bl, kRedThreads, 0, s>>>(a, b, c, n, R, slot);
}

void launch_pcg_direction(cudaStream_t s, double* d, double* zold, const double* z, size_t n,
                          const ReduceScratch& R, int first) {
  k_pcg_direction<<<stride_blocks(n) * 2, kRedThreads, 0, s>>>(d, zold, z, n, R, first);
  k_pcg_keep_rz<<<1, 1, 0, s>>>(R);
}

void launch_pcg_step(cudaStream_t s, double* x, const double* d, size_t n, const ReduceScratch& R) {
  k_pcg_step<<<stride_blocks(n) * 2, kRedThreads, 0, s>>>(x, d, n, R);
}

}  // namespace gbmg
