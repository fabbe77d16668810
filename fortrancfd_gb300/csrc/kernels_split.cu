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
// rho and writes its own half of p, all coalesced.  A sweep's algorithmic
// traffic is 16 bytes per cell (p read and written, b and rho read once); the
// two colour launches read rho twice, 20 bytes per cell, unless the second
// finds the first's rho still in L2.  The kernels here do the arithmetic of the natural-layout kernels
// (k_smooth, k_restrict, k_prolong with the density form) in the same order,
// so both layouts give bit-identical results.
#include <algorithm>
#include <cstdlib>
#include <type_traits>

#include "gbmg_internal.h"
#include "pdl.cuh"

namespace gbmg {

namespace {

inline unsigned cdiv(size_t a, unsigned b) { return (unsigned)((a + b - 1) / b); }

__device__ __forceinline__ float face(float k, float ra, float rb) { return rho_face32(k, ra, rb); }
__device__ __forceinline__ float rho_update(float v, float d) { return rho_update32(v, d); }

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
    if (!kZero) rho_acc32(c, po[tt], s, d);     \
    else d = __fadd_rn(d, c);                   \
  }
  SPLIT_TERM(i > 0, L.kx, h - 1 + par)
  SPLIT_TERM(i < L.nx - 1, L.kx, h + par)
  SPLIT_TERM(j > 0, L.ky, h - sy)
  SPLIT_TERM(j < L.ny - 1, L.ky, h + sy)
  SPLIT_TERM(k > 0, L.kz, h - sz)
  SPLIT_TERM(k < L.nz - 1, L.kz, h + sz)
#undef SPLIT_TERM
  L.sol[own] = rho_relax32(s, L.src[own], d);
}

__device__ __forceinline__ float4 ld4(const float* p) { return *reinterpret_cast<const float4*>(p); }
__device__ __forceinline__ void st4(float* p, float4 v) { *reinterpret_cast<float4*>(p) = v; }
__device__ __forceinline__ void unpack(float4 v, float (&a)[4]) { a[0] = v.x; a[1] = v.y; a[2] = v.z; a[3] = v.w; }

// k_smooth_split with four cells per thread (half indices m0..m0+3 of a row,
// nx % 8 == 0): every load is a float4 except the one-element x edge of the
// window, and the index and bounds work is shared by the four cells.  The
// per-cell arithmetic is k_smooth_split's, in the same order.
template <bool kZero>
__global__ void __launch_bounds__(256) k_smooth_split4(LevelView<float> L, int color) {
  pdl_enter();
  const int hx = L.nx >> 1;
  const int m0 = 4 * (blockIdx.x * blockDim.x + threadIdx.x);
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = L.zrev ? L.nz - 1 - (int)blockIdx.z : (int)blockIdx.z;
  if (m0 >= hx || j >= L.ny) return;
  const size_t sy = (size_t)hx, sz = (size_t)hx * L.ny;
  const size_t h = (size_t)k * sz + (size_t)j * sy + m0;
  const int par = (j + k + color) & 1;
  const float* __restrict__ ro = L.rho + (size_t)(1 - color) * L.hstride + h;
  const float* __restrict__ po = L.sol + (size_t)(1 - color) * L.hstride + h;
  const size_t own = (size_t)color * L.hstride + h;
  float rc[4], b[4];
  unpack(ld4(L.rho + own), rc);
  // b is read once per launch and not by the next one (the other colour):
  // streaming loads, so that the L2 keeps rho and p for the next launch
  unpack(__ldcs(reinterpret_cast<const float4*>(L.src + own)), b);
  // A wall face gets neighbour density +inf, so its coefficient k/(rho + inf)
  // is exactly 0 and the term adds nothing: the faces need no branches.
  const float inf = __int_as_float(0x7f800000);
  // x window: the other colour's half indices m0-1+par .. m0+3+par
  float rxm[4], rxp[4], pxm[4] = {0.f, 0.f, 0.f, 0.f}, pxp[4] = {0.f, 0.f, 0.f, 0.f};
  {
    float rv[4], pv[4] = {0.f, 0.f, 0.f, 0.f};
    unpack(ld4(ro), rv);
    if (!kZero) unpack(ld4(po), pv);
    float re = inf, pe = 0.f;
    if (par) {
      if (m0 + 4 < hx) { re = ro[4]; if (!kZero) pe = po[4]; }
      rxm[0] = rv[0]; rxm[1] = rv[1]; rxm[2] = rv[2]; rxm[3] = rv[3];
      rxp[0] = rv[1]; rxp[1] = rv[2]; rxp[2] = rv[3]; rxp[3] = re;
      pxm[0] = pv[0]; pxm[1] = pv[1]; pxm[2] = pv[2]; pxm[3] = pv[3];
      pxp[0] = pv[1]; pxp[1] = pv[2]; pxp[2] = pv[3]; pxp[3] = pe;
    } else {
      if (m0 > 0) { re = ro[-1]; if (!kZero) pe = po[-1]; }
      rxm[0] = re; rxm[1] = rv[0]; rxm[2] = rv[1]; rxm[3] = rv[2];
      rxp[0] = rv[0]; rxp[1] = rv[1]; rxp[2] = rv[2]; rxp[3] = rv[3];
      pxm[0] = pe; pxm[1] = pv[0]; pxm[2] = pv[1]; pxm[3] = pv[2];
      pxp[0] = pv[0]; pxp[1] = pv[1]; pxp[2] = pv[2]; pxp[3] = pv[3];
    }
  }
  float rym[4] = {inf, inf, inf, inf}, ryp[4] = {inf, inf, inf, inf};
  float rzm[4] = {inf, inf, inf, inf}, rzp[4] = {inf, inf, inf, inf};
  float pym[4] = {}, pyp[4] = {}, pzm[4] = {}, pzp[4] = {};
  if (j > 0) { unpack(ld4(ro - sy), rym); if (!kZero) unpack(ld4(po - sy), pym); }
  if (j < L.ny - 1) { unpack(ld4(ro + sy), ryp); if (!kZero) unpack(ld4(po + sy), pyp); }
  if (k > 0) { unpack(ld4(ro - sz), rzm); if (!kZero) unpack(ld4(po - sz), pzm); }
  if (k < L.nz - 1) { unpack(ld4(ro + sz), rzp); if (!kZero) unpack(ld4(po + sz), pzp); }
  float out[4];
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    float s = 0.f, d = 0.f, cc;
    cc = face(L.kx, rc[c], rxm[c]); if (!kZero) rho_acc32(cc, pxm[c], s, d); else d = __fadd_rn(d, cc);
    cc = face(L.kx, rc[c], rxp[c]); if (!kZero) rho_acc32(cc, pxp[c], s, d); else d = __fadd_rn(d, cc);
    cc = face(L.ky, rc[c], rym[c]); if (!kZero) rho_acc32(cc, pym[c], s, d); else d = __fadd_rn(d, cc);
    cc = face(L.ky, rc[c], ryp[c]); if (!kZero) rho_acc32(cc, pyp[c], s, d); else d = __fadd_rn(d, cc);
    cc = face(L.kz, rc[c], rzm[c]); if (!kZero) rho_acc32(cc, pzm[c], s, d); else d = __fadd_rn(d, cc);
    cc = face(L.kz, rc[c], rzp[c]); if (!kZero) rho_acc32(cc, pzp[c], s, d); else d = __fadd_rn(d, cc);
    out[c] = rho_relax32(s, b[c], d);
  }
  st4(L.sol + own, make_float4(out[0], out[1], out[2], out[3]));
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

// k_restrict_split for W coarse cells per thread (I0..I0+W-1, C.nx % W == 0):
// float4 (W = 4) or float2 (W = 2) loads of each child row, the same per-cell
// arithmetic and order.  W = 2 keeps half the loads live (fewer registers,
// more resident warps).
template <int W, bool kStream = false>
__device__ __forceinline__ void ldw(const float* p, float (&a)[W]) {
  if constexpr (W == 4) {
    unpack(kStream ? __ldcs(reinterpret_cast<const float4*>(p)) : ld4(p), a);
  } else {
    const float2 v = kStream ? __ldcs(reinterpret_cast<const float2*>(p))
                             : *reinterpret_cast<const float2*>(p);
    a[0] = v.x;
    a[1] = v.y;
  }
}

template <int W>
__device__ __forceinline__ void stw(float* p, const float (&a)[W]) {
  if constexpr (W == 4) st4(p, make_float4(a[0], a[1], a[2], a[3]));
  else *reinterpret_cast<float2*>(p) = make_float2(a[0], a[1]);
}

// (four blocks per SM: 64 registers with a 32-byte spill, measured faster
// than 72 registers at three blocks)
template <int W>
__global__ void __launch_bounds__(256, 4) k_restrict_splitv(LevelView<float> F, LevelView<float> C,
                                                            int zero_sol) {
  pdl_enter();
  const int I0 = W * (blockIdx.x * blockDim.x + threadIdx.x);
  const int J = blockIdx.y * blockDim.y + threadIdx.y;
  const int K = F.zrev ? C.nz - 1 - (int)blockIdx.z : (int)blockIdx.z;
  if (I0 >= C.nx || J >= C.ny) return;
  const int hx = F.nx >> 1;
  const size_t half = F.hstride;
  const size_t sy = (size_t)hx, sz = (size_t)hx * F.ny;
  const float inf = __int_as_float(0x7f800000);  // wall neighbour: coefficient exactly 0
  float acc[W] = {};
  for (int dz = 0; dz < F.fz; ++dz)
    for (int dy = 0; dy < F.fy; ++dy) {
      const int j = F.fy * J + dy, k = F.fz * K + dz;
      const int ca = (j + k) & 1;
      const size_t h = (size_t)k * sz + (size_t)j * sy + I0;
      const float* Pa = F.sol + (size_t)ca * half + h;
      const float* Pb = F.sol + (size_t)(1 - ca) * half + h;
      const float* Ra = F.rho + (size_t)ca * half + h;
      const float* Rb = F.rho + (size_t)(1 - ca) * half + h;
      float pa[W], pb[W], ra[W], rb[W], ba[W], bb[W];
      ldw<W>(Pa, pa);
      ldw<W>(Pb, pb);
      ldw<W>(Ra, ra);
      ldw<W>(Rb, rb);
      // b is not read again in this cycle: streaming loads
      ldw<W, true>(F.src + (size_t)ca * half + h, ba);
      ldw<W, true>(F.src + (size_t)(1 - ca) * half + h, bb);
      // x-: cell 2I-1 (b's colour, index I-1); x+ of b: cell 2I+2 (a's colour, I+1)
      float pl_e = 0.f, rl_e = inf, pr_e = 0.f, rr_e = inf;
      if (I0 > 0) { pl_e = Pb[-1]; rl_e = Rb[-1]; }
      if (2 * (I0 + W - 1) + 2 < F.nx) { pr_e = Pa[W]; rr_e = Ra[W]; }
      float pym_a[W] = {}, pym_b[W] = {}, pyp_a[W] = {}, pyp_b[W] = {};
      float pzm_a[W] = {}, pzm_b[W] = {}, pzp_a[W] = {}, pzp_b[W] = {};
      float rym_a[W], rym_b[W], ryp_a[W], ryp_b[W], rzm_a[W], rzm_b[W], rzp_a[W], rzp_b[W];
#pragma unroll
      for (int c = 0; c < W; ++c)
        rym_a[c] = rym_b[c] = ryp_a[c] = ryp_b[c] = rzm_a[c] = rzm_b[c] = rzp_a[c] = rzp_b[c] = inf;
      if (j > 0) {
        ldw<W>(Pb - sy, pym_a); ldw<W>(Pa - sy, pym_b);
        ldw<W>(Rb - sy, rym_a); ldw<W>(Ra - sy, rym_b);
      }
      if (j < F.ny - 1) {
        ldw<W>(Pb + sy, pyp_a); ldw<W>(Pa + sy, pyp_b);
        ldw<W>(Rb + sy, ryp_a); ldw<W>(Ra + sy, ryp_b);
      }
      if (k > 0) {
        ldw<W>(Pb - sz, pzm_a); ldw<W>(Pa - sz, pzm_b);
        ldw<W>(Rb - sz, rzm_a); ldw<W>(Ra - sz, rzm_b);
      }
      if (k < F.nz - 1) {
        ldw<W>(Pb + sz, pzp_a); ldw<W>(Pa + sz, pzp_b);
        ldw<W>(Rb + sz, rzp_a); ldw<W>(Ra + sz, rzp_b);
      }
#pragma unroll
      for (int c = 0; c < W; ++c) {
        const float pl = c == 0 ? pl_e : pb[c - 1], rl = c == 0 ? rl_e : rb[c - 1];
        const float pr = c == W - 1 ? pr_e : pa[c + 1], rr = c == W - 1 ? rr_e : ra[c + 1];
        const float cab = face(F.kx, ra[c], rb[c]);
        {
          float s = 0.f, d = 0.f, cc;
          cc = face(F.kx, ra[c], rl); s += cc * pl; d += cc;
          cc = cab; s += cc * pb[c]; d += cc;
          cc = face(F.ky, ra[c], rym_a[c]); s += cc * pym_a[c]; d += cc;
          cc = face(F.ky, ra[c], ryp_a[c]); s += cc * pyp_a[c]; d += cc;
          cc = face(F.kz, ra[c], rzm_a[c]); s += cc * pzm_a[c]; d += cc;
          cc = face(F.kz, ra[c], rzp_a[c]); s += cc * pzp_a[c]; d += cc;
          acc[c] += ba[c] - (s - d * pa[c]);
        }
        {
          float s = 0.f, d = 0.f, cc;
          cc = cab; s += cc * pa[c]; d += cc;
          cc = face(F.kx, rb[c], rr); s += cc * pr; d += cc;
          cc = face(F.ky, rb[c], rym_b[c]); s += cc * pym_b[c]; d += cc;
          cc = face(F.ky, rb[c], ryp_b[c]); s += cc * pyp_b[c]; d += cc;
          cc = face(F.kz, rb[c], rzm_b[c]); s += cc * pzm_b[c]; d += cc;
          cc = face(F.kz, rb[c], rzp_b[c]); s += cc * pzp_b[c]; d += cc;
          acc[c] += bb[c] - (s - d * pb[c]);
        }
      }
    }
  const size_t cq = ((size_t)K * C.ny + J) * C.nx + I0;
  const float sc = 1.f / (float)(F.fx * F.fy * F.fz);
  float out[W], zero[W];
#pragma unroll
  for (int c = 0; c < W; ++c) {
    out[c] = acc[c] * sc;
    zero[c] = 0.f;
  }
  stw<W>(C.src + cq, out);
  if (zero_sol) stw<W>(C.sol + cq, zero);
}

// k_prolong_split for four coarse cells per thread (C.nx % 4 == 0).
// live >= 0: only the cells of that colour are corrected (the other colour is
// overwritten, unread, by the next sweep's first colour launch).
__global__ void __launch_bounds__(256) k_prolong_split4(LevelView<float> F, LevelView<float> C,
                                                        int live) {
  pdl_enter();
  const int I0 = 4 * (blockIdx.x * blockDim.x + threadIdx.x);
  const int J = blockIdx.y * blockDim.y + threadIdx.y;
  const int K = F.zrev ? C.nz - 1 - (int)blockIdx.z : (int)blockIdx.z;
  if (I0 >= C.nx || J >= C.ny) return;
  const size_t csy = (size_t)C.nx, csz = (size_t)C.nx * C.ny;
  const size_t cq = (size_t)K * csz + (size_t)J * csy + I0;
  const float* e = C.sol + cq;
  float ec[4], eym[4], eyp[4], ezm[4], ezp[4];
  unpack(ld4(e), ec);
  const float el = I0 > 0 ? e[-1] : ec[0];
  const float er = I0 + 4 < C.nx ? e[4] : ec[3];
  float mx[4], my[4] = {0.f, 0.f, 0.f, 0.f}, mz[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    const float hi = c == 3 ? er : ec[c + 1];
    const float lo = c == 0 ? el : ec[c - 1];
    mx[c] = 0.5f * (hi - lo);
  }
  if (F.fy == 2) {
    if (J < C.ny - 1) unpack(ld4(e + csy), eyp); else unpack(ld4(e), eyp);
    if (J > 0) unpack(ld4(e - csy), eym); else unpack(ld4(e), eym);
#pragma unroll
    for (int c = 0; c < 4; ++c) my[c] = 0.5f * (eyp[c] - eym[c]);
  }
  if (F.fz == 2) {
    if (K < C.nz - 1) unpack(ld4(e + csz), ezp); else unpack(ld4(e), ezp);
    if (K > 0) unpack(ld4(e - csz), ezm); else unpack(ld4(e), ezm);
#pragma unroll
    for (int c = 0; c < 4; ++c) mz[c] = 0.5f * (ezp[c] - ezm[c]);
  }
  const int hx = F.nx >> 1;
  const size_t half = F.hstride;
  for (int dz = 0; dz < F.fz; ++dz)
    for (int dy = 0; dy < F.fy; ++dy) {
      const int j = F.fy * J + dy, k = F.fz * K + dz;
      const int ca = (j + k) & 1;
      const size_t h = ((size_t)k * F.ny + j) * hx + I0;
      float* A = F.sol + (size_t)ca * half + h;
      float* B = F.sol + (size_t)(1 - ca) * half + h;
      const bool da = live < 0 || live == ca, db = live < 0 || live != ca;
      float a[4], b[4];
      if (da) unpack(ld4(A), a);
      if (db) unpack(ld4(B), b);
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const float ty = dy ? 0.25f * my[c] : -(0.25f * my[c]);
        const float tz = dz ? 0.25f * mz[c] : -(0.25f * mz[c]);
        float v0 = ec[c] + -(0.25f * mx[c]), v1 = ec[c] + 0.25f * mx[c];
        if (F.fy == 2) { v0 += ty; v1 += ty; }
        if (F.fz == 2) { v0 += tz; v1 += tz; }
        a[c] += v0;
        b[c] += v1;
      }
      if (da) st4(A, make_float4(a[0], a[1], a[2], a[3]));
      if (db) st4(B, make_float4(b[0], b[1], b[2], b[3]));
    }
}

// Prolongation + correction into the split finest level (fx = 2), as k_prolong
// (live: as in k_prolong_split4).
__global__ void __launch_bounds__(256) k_prolong_split(LevelView<float> F, LevelView<float> C,
                                                       int live) {
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
      if (live < 0 || live == ca) F.sol[(size_t)ca * half + h] += v0;
      if (live < 0 || live != ca) F.sol[(size_t)(1 - ca) * half + h] += v1;
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

// the four-cell kernels need rows of whole float4 groups in each half
inline bool vec4_ok(const LevelView<float>& F) {
  return F.nx % 8 == 0 && F.hstride % 4 == 0;
}

void launch_smooth_split(cudaStream_t s, const LevelView<float>& L, int color, bool zero_guess) {
  const dim3 blk(32, 8, 1);
  if (vec4_ok(L)) {
    const dim3 g4(cdiv((size_t)(L.nx / 8), 32), cdiv((size_t)L.ny, 8), (unsigned)L.nz);
    if (zero_guess) launch_pdl(k_smooth_split4<true>, g4, blk, 0, s, L, color);
    else launch_pdl(k_smooth_split4<false>, g4, blk, 0, s, L, color);
    return;
  }
  const dim3 grd(cdiv((size_t)(L.nx / 2), 32), cdiv((size_t)L.ny, 8), (unsigned)L.nz);
  if (zero_guess) launch_pdl(k_smooth_split<true>, grd, blk, 0, s, L, color);
  else launch_pdl(k_smooth_split<false>, grd, blk, 0, s, L, color);
}

void launch_restrict_split(cudaStream_t s, const LevelView<float>& F, const LevelView<float>& C,
                           bool zero_sol) {
  const dim3 blk(32, 8, 1);
  if (vec4_ok(F) && C.nx % 4 == 0) {
    // two coarse cells per thread
    const dim3 gv(cdiv((size_t)(C.nx / 2), 32), cdiv((size_t)C.ny, 8), (unsigned)C.nz);
    launch_pdl(k_restrict_splitv<2>, gv, blk, 0, s, F, C, zero_sol ? 1 : 0);
    return;
  }
  const dim3 grd(cdiv((size_t)C.nx, 32), cdiv((size_t)C.ny, 8), (unsigned)C.nz);
  launch_pdl(k_restrict_split, grd, blk, 0, s, F, C, zero_sol ? 1 : 0);
}

void launch_prolong_split(cudaStream_t s, const LevelView<float>& F, const LevelView<float>& C,
                          int live) {
  const dim3 blk(32, 8, 1);
  if (vec4_ok(F) && C.nx % 4 == 0) {
    const dim3 g4(cdiv((size_t)(C.nx / 4), 32), cdiv((size_t)C.ny, 8), (unsigned)C.nz);
    launch_pdl(k_prolong_split4, g4, blk, 0, s, F, C, live);
    return;
  }
  const dim3 grd(cdiv((size_t)C.nx, 32), cdiv((size_t)C.ny, 8), (unsigned)C.nz);
  launch_pdl(k_prolong_split, grd, blk, 0, s, F, C, live);
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
