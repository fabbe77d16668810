// Colour-split layout of the FP32 finest level (sm_103a).
//
// A red-black sweep in the natural layout moves every array in full 32-byte
// sectors in both colour launches, although each launch needs only half of
// p, b and the writes: 2 x 16 bytes per cell per sweep with the density-form
// coefficients.  In the colour-split layout each FP32 finest-level array
// (p, b, rho) holds the cells of colour 0 ((i+j+k) even) in its first half
// and those of colour 1 in its second half, each half in natural order with
// x halved: cell (i, j, k) lives at
//     ((i + j + k) & 1) * hstride + ((k*ny + j)*nx + i)/2        (nx even),
// hstride = n/2 plus a small pad, so that the halves do not sit a power of two
// apart (same-offset accesses to both halves would fall on the same DRAM
// channels).
// All six neighbours of a cell are of the other colour, at half-index offsets
// -1/0 or 0/+1 (x, by the cell's parity), -+nx/2 (y) and -+nx*ny/2 (z), so a
// colour launch reads the other half of p and rho and its own half of b and
// rho and writes its own half of p, all coalesced: 20 bytes per cell per
// sweep.  The kernels here do the arithmetic of the natural-layout kernels
// (k_smooth, k_restrict, k_prolong with the density form) in the same order,
// so both layouts give bit-identical results.
#include <type_traits>

#include "gbmg_internal.h"
#include "pdl.cuh"

namespace gbmg {

namespace {

inline unsigned cdiv(size_t a, unsigned b) { return (unsigned)((a + b - 1) / b); }

__device__ __forceinline__ float face(float k, float ra, float rb) { return __fdividef(k, ra + rb); }

// One colour of a red-black sweep, one thread per cell of the colour.
template <bool kZero>
__global__ void __launch_bounds__(256) k_smooth_split(LevelView<float> L, int color) {
  pdl_enter();
  const int hx = L.nx >> 1;
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (m >= hx || j >= L.ny) return;
  const size_t half = L.hstride;
  const size_t sy = (size_t)hx, sz = (size_t)hx * L.ny;
  const size_t h = (size_t)k * sz + (size_t)j * sy + m;
  const int par = (j + k + color) & 1;
  const int i = 2 * m + par;
  const float* __restrict__ ro = L.rho + (size_t)(1 - color) * half;
  const float* __restrict__ po = L.sol + (size_t)(1 - color) * half;
  const size_t own = (size_t)color * half + h;
  const float rc = L.rho[own];
  float s = 0.f, d = 0.f, c;
#define SPLIT_TERM(cond, kk, t)                 \
  if (cond) {                                   \
    const size_t tt = (t);                      \
    c = face(kk, rc, ro[tt]);                   \
    if (!kZero) s += c * po[tt];                \
    d += c;                                     \
  }
  SPLIT_TERM(i > 0, L.kx, h - 1 + par)
  SPLIT_TERM(i < L.nx - 1, L.kx, h + par)
  SPLIT_TERM(j > 0, L.ky, h - sy)
  SPLIT_TERM(j < L.ny - 1, L.ky, h + sy)
  SPLIT_TERM(k > 0, L.kz, h - sz)
  SPLIT_TERM(k < L.nz - 1, L.kz, h + sz)
#undef SPLIT_TERM
  const float v = s - L.src[own];
  L.sol[own] = v / d;
}

// Fused residual + restriction out of the split finest level (fx = 2): one
// thread per coarse cell; per child row the children x = 2I (colour ca) and
// x = 2I+1 (colour 1-ca) share the half index of the row plus I.
__global__ void __launch_bounds__(256) k_restrict_split(LevelView<float> F, LevelView<float> C,
                                                        int zero_sol) {
  pdl_enter();
  const int I = blockIdx.x * blockDim.x + threadIdx.x;
  const int J = blockIdx.y * blockDim.y + threadIdx.y;
  const int K = blockIdx.z;
  if (I >= C.nx || J >= C.ny) return;
  const int hx = F.nx >> 1;
  const size_t half = F.hstride;
  const size_t sy = (size_t)hx, sz = (size_t)hx * F.ny;
  float acc = 0.f;
  for (int dz = 0; dz < F.fz; ++dz)
    for (int dy = 0; dy < F.fy; ++dy) {
      const int j = F.fy * J + dy, k = F.fz * K + dz;
      const int ca = (j + k) & 1;
      const size_t h = (size_t)k * sz + (size_t)j * sy + I;
      const float* Pa = F.sol + (size_t)ca * half;        // colour of child a
      const float* Pb = F.sol + (size_t)(1 - ca) * half;  // colour of child b
      const float* Ra = F.rho + (size_t)ca * half;
      const float* Rb = F.rho + (size_t)(1 - ca) * half;
      const float* Ba = F.src + (size_t)ca * half;
      const float* Bb = F.src + (size_t)(1 - ca) * half;
      const bool xl = 2 * I > 0, xr = 2 * I + 2 < F.nx;
      const bool yl = j > 0, yr = j < F.ny - 1, zl = k > 0, zr = k < F.nz - 1;
      const float pa = Pa[h], pb = Pb[h], ra = Ra[h], rb = Rb[h];
      // x-: cell 2I-1 (colour of b, index h-1); x+ of b: cell 2I+2 (colour of a, h+1)
      const float pl = xl ? Pb[h - 1] : 0.f, pr = xr ? Pa[h + 1] : 0.f;
      // y/z neighbours of a have b's colour and vice versa
      const float pym_a = yl ? Pb[h - sy] : 0.f, pym_b = yl ? Pa[h - sy] : 0.f;
      const float pyp_a = yr ? Pb[h + sy] : 0.f, pyp_b = yr ? Pa[h + sy] : 0.f;
      const float pzm_a = zl ? Pb[h - sz] : 0.f, pzm_b = zl ? Pa[h - sz] : 0.f;
      const float pzp_a = zr ? Pb[h + sz] : 0.f, pzp_b = zr ? Pa[h + sz] : 0.f;
      const float cxa = xl ? face(F.kx, ra, Rb[h - 1]) : 0.f;
      const float cab = face(F.kx, ra, rb);
      const float cxr = xr ? face(F.kx, rb, Ra[h + 1]) : 0.f;
      const float cym_a = yl ? face(F.ky, ra, Rb[h - sy]) : 0.f;
      const float cym_b = yl ? face(F.ky, rb, Ra[h - sy]) : 0.f;
      const float cyp_a = yr ? face(F.ky, ra, Rb[h + sy]) : 0.f;
      const float cyp_b = yr ? face(F.ky, rb, Ra[h + sy]) : 0.f;
      const float czm_a = zl ? face(F.kz, ra, Rb[h - sz]) : 0.f;
      const float czm_b = zl ? face(F.kz, rb, Ra[h - sz]) : 0.f;
      const float czp_a = zr ? face(F.kz, ra, Rb[h + sz]) : 0.f;
      const float czp_b = zr ? face(F.kz, rb, Ra[h + sz]) : 0.f;
      {
        float s = 0.f, d = 0.f, c;
        if (xl) { c = cxa; s += c * pl; d += c; }
        c = cab; s += c * pb; d += c;
        if (yl) { c = cym_a; s += c * pym_a; d += c; }
        if (yr) { c = cyp_a; s += c * pyp_a; d += c; }
        if (zl) { c = czm_a; s += c * pzm_a; d += c; }
        if (zr) { c = czp_a; s += c * pzp_a; d += c; }
        acc += Ba[h] - (s - d * pa);
      }
      {
        float s = 0.f, d = 0.f, c;
        c = cab; s += c * pa; d += c;
        if (xr) { c = cxr; s += c * pr; d += c; }
        if (yl) { c = cym_b; s += c * pym_b; d += c; }
        if (yr) { c = cyp_b; s += c * pyp_b; d += c; }
        if (zl) { c = czm_b; s += c * pzm_b; d += c; }
        if (zr) { c = czp_b; s += c * pzp_b; d += c; }
        acc += Bb[h] - (s - d * pb);
      }
    }
  const size_t cq = ((size_t)K * C.ny + J) * C.nx + I;
  C.src[cq] = acc * (1.f / (float)(F.fx * F.fy * F.fz));
  if (zero_sol) C.sol[cq] = 0.f;
}

// Prolongation + correction into the split finest level (fx = 2), as k_prolong.
__global__ void __launch_bounds__(256) k_prolong_split(LevelView<float> F, LevelView<float> C) {
  pdl_enter();
  const int I = blockIdx.x * blockDim.x + threadIdx.x;
  const int J = blockIdx.y * blockDim.y + threadIdx.y;
  const int K = blockIdx.z;
  if (I >= C.nx || J >= C.ny) return;
  const size_t csy = (size_t)C.nx, csz = (size_t)C.nx * C.ny;
  const size_t cq = (size_t)K * csz + (size_t)J * csy + I;
  const float* e = C.sol;
  const float ec = e[cq];
  float mx = 0.f, my = 0.f, mz = 0.f;
  mx = 0.5f * ((I < C.nx - 1 ? e[cq + 1] : ec) - (I > 0 ? e[cq - 1] : ec));
  if (F.fy == 2) my = 0.5f * ((J < C.ny - 1 ? e[cq + csy] : ec) - (J > 0 ? e[cq - csy] : ec));
  if (F.fz == 2) mz = 0.5f * ((K < C.nz - 1 ? e[cq + csz] : ec) - (K > 0 ? e[cq - csz] : ec));
  const int hx = F.nx >> 1;
  const size_t half = F.hstride;
  for (int dz = 0; dz < F.fz; ++dz)
    for (int dy = 0; dy < F.fy; ++dy) {
      const int j = F.fy * J + dy, k = F.fz * K + dz;
      const int ca = (j + k) & 1;
      const size_t h = ((size_t)k * F.ny + j) * hx + I;
      const float ty = dy ? 0.25f * my : -(0.25f * my);
      const float tz = dz ? 0.25f * mz : -(0.25f * mz);
      float v0 = ec + -(0.25f * mx), v1 = ec + 0.25f * mx;
      if (F.fy == 2) { v0 += ty; v1 += ty; }
      if (F.fz == 2) { v0 += tz; v1 += tz; }
      F.sol[(size_t)ca * half + h] += v0;
      F.sol[(size_t)(1 - ca) * half + h] += v1;
    }
}

// double (natural) -> float (split), and float (split) -> double (natural)
__global__ void k_to_split(const double* __restrict__ a, float* __restrict__ out, int nx, int ny,
                           int nz, size_t half) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i >= nx || j >= ny) return;
  const size_t q = ((size_t)k * ny + j) * nx + i;
  out[(size_t)((i + j + k) & 1) * half + (q >> 1)] = (float)a[q];
}

__global__ void k_from_split(const float* __restrict__ a, double* __restrict__ out, int nx, int ny,
                             int nz, size_t half) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i >= nx || j >= ny) return;
  const size_t q = ((size_t)k * ny + j) * nx + i;
  out[q] = (double)a[(size_t)((i + j + k) & 1) * half + (q >> 1)];
}

}  // namespace

void launch_smooth_split(cudaStream_t s, const LevelView<float>& L, int color, bool zero_guess) {
  const dim3 blk(32, 8, 1);
  const dim3 grd(cdiv((size_t)(L.nx / 2), 32), cdiv((size_t)L.ny, 8), (unsigned)L.nz);
  if (zero_guess) launch_pdl(k_smooth_split<true>, grd, blk, 0, s, L, color);
  else launch_pdl(k_smooth_split<false>, grd, blk, 0, s, L, color);
}

void launch_restrict_split(cudaStream_t s, const LevelView<float>& F, const LevelView<float>& C,
                           bool zero_sol) {
  const dim3 blk(32, 8, 1);
  const dim3 grd(cdiv((size_t)C.nx, 32), cdiv((size_t)C.ny, 8), (unsigned)C.nz);
  launch_pdl(k_restrict_split, grd, blk, 0, s, F, C, zero_sol ? 1 : 0);
}

void launch_prolong_split(cudaStream_t s, const LevelView<float>& F, const LevelView<float>& C) {
  const dim3 blk(32, 8, 1);
  const dim3 grd(cdiv((size_t)C.nx, 32), cdiv((size_t)C.ny, 8), (unsigned)C.nz);
  launch_pdl(k_prolong_split, grd, blk, 0, s, F, C);
}

void launch_to_split(cudaStream_t s, const double* a, float* out, int nx, int ny, int nz,
                     size_t hstride) {
  const dim3 blk(32, 8, 1);
  const dim3 grd(cdiv((size_t)nx, 32), cdiv((size_t)ny, 8), (unsigned)nz);
  k_to_split<<<grd, blk, 0, s>>>(a, out, nx, ny, nz, hstride);
}

void launch_from_split(cudaStream_t s, const float* a, double* out, int nx, int ny, int nz,
                       size_t hstride) {
  const dim3 blk(32, 8, 1);
  const dim3 grd(cdiv((size_t)nx, 32), cdiv((size_t)ny, 8), (unsigned)nz);
  k_from_split<<<grd, blk, 0, s>>>(a, out, nx, ny, nz, hstride);
}

}  // namespace gbmg
