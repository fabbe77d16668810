// Double-word kernels of the mixed-precision solve (sm_103a).
//
// k_defect is the FP64-accuracy half of one defect-correction step:
//     p_out = p_in + e          (e: the FP32 V-cycle's correction)
//     r     = b - A p_out       (the operator of ppe_sor_init, double-word)
//     r32   = float(r), and sum r^2 for the stopping test
// in one pass.  Blocks own 32 x 8 tiles of the x-y plane and march up a chunk
// of z planes with a 3-plane ring of p_out (tile + 1-cell halo) in shared
// memory; halo cells are updated redundantly and only the owner stores them.
// It runs out of place (p_in -> p_out) so that no block ever reads a value
// another block already advanced.  Per cell: read p (8 B), e (4), b (8), three
// coefficients (24); write p (8), r32 (4): 56 bytes.
//
// The residual is sum_f coe_f (p_nb - p_i) as in multigrid_residual
// ("DomainDecomposition/3D/src/others/multigrid_solver.f90:162-222") with the
// coefficients of ppe_sor_init ("Two phase flows/newOpenMP/3D+IBM/src/
// ns_solver/ns_ppe_solver.f90:1-65"): differences first, so each term's
// rounding is relative to a flux, not to |p|.
#include <cudaTypedefs.h>

#include <algorithm>

#include "dword.cuh"
#include "gbmg_internal.h"
#include "pdl.cuh"
#include "reduce.cuh"
#include "tma.cuh"

namespace gbmg {

namespace {

constexpr int kDTX = 32, kDTY = 8, kDZ = 32;
constexpr int kDSX = kDTX + 2, kDSY = kDTY + 2;

struct DefectRing {
  float2 p[3][kDSY][kDSX];
};

// Index of natural cell q = (k, y, x) in an FP32 finest-level array: the
// natural index (hstride 0), or the colour-split one ((x+y+k)&1)*hstride + q/2.
__device__ __forceinline__ size_t fine_index(size_t q, int x, int y, int k, size_t hstride) {
  return hstride ? (size_t)((x + y + k) & 1) * hstride + (q >> 1) : q;
}

__device__ __forceinline__ void defect_load(const DwOperator& A, const float2* __restrict__ pin,
                                            float2* __restrict__ pout, const float* __restrict__ e,
                                            DefectRing& R, int k, int x0, int y0, int z0, int z1,
                                            int tid, size_t hstride) {
  const int slot = k % 3;
  const size_t sz = (size_t)A.nx * A.ny;
  for (int t = tid; t < kDSX * kDSY; t += kDTX * kDTY) {
    const int lx = t % kDSX, ly = t / kDSX;
    const int x = x0 - 1 + lx, y = y0 - 1 + ly;
    float2 v = make_float2(0.f, 0.f);
    if (x >= 0 && x < A.nx && y >= 0 && y < A.ny) {
      const size_t q = (size_t)k * sz + (size_t)y * A.nx + x;
      dw a = dw_ldg(pin + q);
      if (e) a = dw_add_f(a, __ldg(e + fine_index(q, x, y, k, hstride)));
      v = make_float2(a.hi, a.lo);
      if (lx >= 1 && lx <= kDTX && ly >= 1 && ly <= kDTY && k >= z0 && k < z1) pout[q] = v;
    }
    R.p[slot][ly][lx] = v;
  }
}

__global__ void __launch_bounds__(kDTX * kDTY) k_defect(DwOperator A, const float2* __restrict__ pin,
                                                        float2* __restrict__ pout,
                                                        const float* __restrict__ e,
                                                        float* __restrict__ r32, ReduceScratch R,
                                                        int slot, size_t hstride) {
  pdl_enter();
  __shared__ DefectRing ring;
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * kDTX + tx;
  const int x0 = blockIdx.x * kDTX, y0 = blockIdx.y * kDTY;
  const int z0 = blockIdx.z * kDZ, z1 = min(z0 + kDZ, A.nz);
  const int x = x0 + tx, y = y0 + ty;
  const bool mine = x < A.nx && y < A.ny;
  const size_t sy = (size_t)A.nx, sz = (size_t)A.nx * A.ny;
  float s2 = 0.f;
  if (z0 > 0) defect_load(A, pin, pout, e, ring, z0 - 1, x0, y0, z0, z1, tid, hstride);
  defect_load(A, pin, pout, e, ring, z0, x0, y0, z0, z1, tid, hstride);
  for (int k = z0; k < z1; ++k) {
    if (k + 1 < A.nz) defect_load(A, pin, pout, e, ring, k + 1, x0, y0, z0, z1, tid, hstride);
    __syncthreads();
    if (mine) {
      const int s0 = k % 3, sm = (k + 2) % 3, sp = (k + 1) % 3;
      const size_t q = (size_t)k * sz + (size_t)y * sy + x;
      const float2 c2 = ring.p[s0][ty + 1][tx + 1];
      const dw pc{c2.x, c2.y};
      residual_acc acc(dw_ldg(A.b + q));
#define DW_TERM(cond, cptr, nbv)                                   \
      if (cond) {                                                  \
        const float2 nb = nbv;                                     \
        acc.sub(flux_term(dw_ldg(cptr), dw{nb.x, nb.y}, pc));      \
      }
      DW_TERM(x > 0, A.cx + q, ring.p[s0][ty + 1][tx])
      DW_TERM(x < A.nx - 1, A.cx + q + 1, ring.p[s0][ty + 1][tx + 2])
      DW_TERM(y > 0, A.cy + q, ring.p[s0][ty][tx + 1])
      DW_TERM(y < A.ny - 1, A.cy + q + sy, ring.p[s0][ty + 2][tx + 1])
      DW_TERM(k > 0, A.cz + q, ring.p[sm][ty + 1][tx + 1])
      DW_TERM(k < A.nz - 1, A.cz + q + sz, ring.p[sp][ty + 1][tx + 1])
#undef DW_TERM
      const float rf = acc.value_f();
      r32[fine_index(q, x, y, k, hstride)] = rf;
      s2 = fmaf(rf, rf, s2);
    }
    __syncthreads();
  }
  double v[1] = {(double)s2};
  grid_sum_finish<1>(v, R, slot);
}

// ---- TMA-fed defect ------------------------------------------------------------
// Same arithmetic as k_defect; each plane's boxes (tile + 1-cell halo) of p, b,
// cx, cy, cz (float pairs, through FP32 maps of doubled x extent, box from
// x0-2) and e (FP32, box from x0-4) stream into a 4-slot ring two planes ahead
// of the compute.  With the colour-split finest level, e comes as two boxes
// (its colour-0 and colour-1 planes, x halved, box from x0/2-4) out of two
// maps, one per colour half.  Wall coefficients are stored as zeros and TMA zero-fills
// out-of-range box cells, so x and y walls add exact zeros.
constexpr int kQBX = kDTX + 4;         // float-pair box width, from x0 - 2
constexpr int kQBY = kDTY + 2;         // box height, from y0 - 1
constexpr int kQEX = kDTX + 8;         // e box width, from x0 - 4
constexpr int kQSEX = kDTX / 2 + 8;    // split e box width, from x0/2 - 4
constexpr int kQSEOff = 256;           // floats from the colour-0 to the colour-1 split box
constexpr int kQSlots = 4;
constexpr int kQTile = kQBX * kQBY;    // float pairs per box (2880 bytes)
constexpr int kQTileBytes = 2944;      // padded to a multiple of 128
constexpr int kQEBytes = 2048;         // e box (1600 bytes), or the two split boxes at 0 and 1024
constexpr int kQSlotBytes = 5 * kQTileBytes + kQEBytes;  // 16384
constexpr uint32_t kQPairBytes = kQTile * 8;
constexpr uint32_t kQEBoxBytes = kQEX * kQBY * 4;
constexpr uint32_t kQSEBoxBytes = kQSEX * kQBY * 4;
constexpr size_t kQSmem = (size_t)kQSlots * kQSlotBytes + 128 + kQSlots * sizeof(uint64_t);

__device__ __forceinline__ float2* qtile(unsigned char* base, int slot, int a) {
  return reinterpret_cast<float2*>(base + (size_t)slot * kQSlotBytes + (size_t)a * kQTileBytes);
}
__device__ __forceinline__ float* qtile_e(unsigned char* base, int slot) {
  return reinterpret_cast<float*>(base + (size_t)slot * kQSlotBytes + 5 * kQTileBytes);
}

__global__ void __launch_bounds__(kDTX * kDTY, 3)
    k_defect_tma(const __grid_constant__ DefectMaps maps, int nx, int ny, int nz, int use_e,
                 float2* __restrict__ pout, float* __restrict__ r32, ReduceScratch R, int slot,
                 int* err, size_t hstride) {
  pdl_enter();
  const bool split = hstride != 0;
  extern __shared__ unsigned char dsm_raw[];
  unsigned char* base =
      reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(dsm_raw) + 127) & ~uintptr_t(127));
  uint64_t* bar = reinterpret_cast<uint64_t*>(base + (size_t)kQSlots * kQSlotBytes);
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * kDTX + tx;
  const int x0 = blockIdx.x * kDTX, y0 = blockIdx.y * kDTY;
  const int z0 = blockIdx.z * kDZ, z1 = min(z0 + kDZ, nz);
  const int plo = max(z0 - 1, 0), phi = min(z1, nz - 1);
  if (tid == 0) {
    for (int s = 0; s < kQSlots; ++s) mbar_init(&bar[s], 1);
    fence_barrier_init();
  }
  __syncthreads();
  auto issue = [&](int k) {  // thread 0
    const int s = k % kQSlots;
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    const uint32_t ebytes = use_e ? (split ? 2 * kQSEBoxBytes : kQEBoxBytes) : 0;
    mbar_arrive_expect_tx(&bar[s], 5 * kQPairBytes + ebytes);
    const int xq = 2 * (x0 - 2), yq = y0 - 1;
    tma_load_3d(qtile(base, s, 0), &maps.p, xq, yq, k, &bar[s]);
    tma_load_3d(qtile(base, s, 1), &maps.b, xq, yq, k, &bar[s]);
    tma_load_3d(qtile(base, s, 2), &maps.cx, xq, yq, k, &bar[s]);
    tma_load_3d(qtile(base, s, 3), &maps.cy, xq, yq, k, &bar[s]);
    tma_load_3d(qtile(base, s, 4), &maps.cz, xq, yq, k, &bar[s]);
    if (use_e && split) {
      tma_load_3d(qtile_e(base, s), &maps.e, (x0 >> 1) - 4, yq, k, &bar[s]);
      tma_load_3d(qtile_e(base, s) + kQSEOff, &maps.e1, (x0 >> 1) - 4, yq, k, &bar[s]);
    } else if (use_e) {
      tma_load_3d(qtile_e(base, s), &maps.e, x0 - 4, yq, k, &bar[s]);
    }
  };
  // this thread's box cells for the p + e update (at most two: the box has
  // kQTile cells for kDTX * kDTY threads), with their e offsets worked out
  // once: the split e box holds a cell of parity c at c * kQSEOff + its row's
  // offset, and the parity of box cell (x, y) flips with every plane
  constexpr int kBoxPer = (kQTile + kDTX * kDTY - 1) / (kDTX * kDTY);
  static_assert(kBoxPer == 2, "two box cells per thread");
  int boff[kBoxPer], eoff[kBoxPer], bpar[kBoxPer];
#pragma unroll
  for (int u = 0; u < kBoxPer; ++u) {
    const int t = tid + u * kDTX * kDTY;
    boff[u] = t < kQTile ? t : -1;
    const int row = t / kQBX, col = t % kQBX;
    const int xx = x0 - 2 + col, yy = y0 - 1 + row;
    eoff[u] = split ? row * kQSEX + ((xx >> 1) - (x0 >> 1) + 4) : row * kQEX + col + 2;
    bpar[u] = (xx + yy) & 1;
  }
  uint32_t parity = 0;
  const int pre_end = min(z0 + 1, phi);
  if (tid == 0)
    for (int k = plo; k <= pre_end; ++k) issue(k);
  int issued = pre_end, waited = plo - 1;
  float s2 = 0.f;
  dw fz_carry{0.f, 0.f};  // z flux between planes k-1 and k, computed at plane k-1
  for (int k = z0; k < z1; ++k) {
    if (k + 2 <= phi && k + 2 > issued) {
      if (tid == 0) issue(k + 2);
      issued = k + 2;
    }
    const int need = min(k + 1, phi);
    while (waited < need) {
      ++waited;
      const int s = waited % kQSlots;
      mbar_wait(&bar[s], (parity >> s) & 1u, err);
      parity ^= 1u << s;
      if (use_e) {  // p + e on the whole box
        float2* P = qtile(base, s, 0);
        const float* E = qtile_e(base, s);
#pragma unroll
        for (int u = 0; u < kBoxPer; ++u) {
          const int t = boff[u];
          if (t < 0) continue;
          // box cell (row, col) is x = x0-2+col, y = y0-1+row of plane `waited`
          const float ev = E[split ? ((bpar[u] + waited) & 1) * kQSEOff + eoff[u] : eoff[u]];
          const float2 pv = P[t];
          const dw a = dw_add_f(dw{pv.x, pv.y}, ev);
          P[t] = make_float2(a.hi, a.lo);
        }
      }
      __syncthreads();
    }
    // Face terms in the order x-, x+, y-, y+, z-, z+; the z- term is the
    // previous plane's z+ term negated (flux_term is sign-symmetric, so this
    // is bit-identical to computing it), except at the first plane of the
    // chunk.
    {
      const int x = x0 + tx, y = y0 + ty;
      const int s0 = k % kQSlots, sm = (k + kQSlots - 1) % kQSlots, sp = (k + 1) % kQSlots;
      const int t = (ty + 1) * kQBX + (tx + 2);
      const float2* P = qtile(base, s0, 0);
      const float2* CX = qtile(base, s0, 2);
      const float2* CY = qtile(base, s0, 3);
      const float2 pc2 = P[t];
      const dw pc{pc2.x, pc2.y};
      const auto ld = [](const float2* a, int i) { const float2 v = a[i]; return dw{v.x, v.y}; };
      const dw fxm = flux_term(ld(CX, t), ld(P, t - 1), pc);  // c (p_{x-1} - p_c)
      const dw fxp = flux_term(ld(CX, t + 1), ld(P, t + 1), pc);
      const dw fym = flux_term(ld(CY, t), ld(P, t - kQBX), pc);
      const dw fyp = flux_term(ld(CY, t + kQBX), ld(P, t + kQBX), pc);
      dw fzm{0.f, 0.f}, fzp{0.f, 0.f};
      if (k > 0) {
        if (k == z0) fzm = flux_term(ld(qtile(base, s0, 4), t), ld(qtile(base, sm, 0), t), pc);
        else fzm = dw{-fz_carry.hi, -fz_carry.lo};
      }
      if (k < nz - 1) fzp = flux_term(ld(qtile(base, sp, 4), t), ld(qtile(base, sp, 0), t), pc);
      fz_carry = fzp;
      if (x < nx && y < ny) {
        const float2 b2 = qtile(base, s0, 1)[t];
        residual_acc acc(dw{b2.x, b2.y});
        acc.sub(fxm);
        acc.sub(fxp);
        acc.sub(fym);
        acc.sub(fyp);
        if (k > 0) acc.sub(fzm);
        if (k < nz - 1) acc.sub(fzp);
        const size_t q = ((size_t)k * ny + y) * nx + x;
        const float rf = acc.value_f();
        r32[fine_index(q, x, y, k, hstride)] = rf;
        pout[q] = pc2;
        s2 = fmaf(rf, rf, s2);
      }
    }
    __syncthreads();
  }
  double v[1] = {(double)s2};
  grid_sum_finish<1>(v, R, slot);
}

__global__ void k_to_dw(const double* __restrict__ a, float2* __restrict__ out, size_t n) {
  stride4(n, [&](size_t q) { return a[q]; }, [&](size_t q, double x) {
    const dw v = dw_from_double_int(x);
    out[q] = make_float2(v.hi, v.lo);
  });
}

// slot <- sum of the values of p (for the final mean projection): each
// thread sums its elements in double-word on the FP32 pipes (error about
// 2u^2 of the partial sums, u = 2^-24), the threads' sums are added in FP64
__global__ void __launch_bounds__(kRedThreads) k_dw_sum(const float2* __restrict__ p, size_t n,
                                                        ReduceScratch R, int slot) {
  dw a{0.f, 0.f};
  stride4(n, [&](size_t q) { return dw_ldg(p + q); }, [&](size_t, dw v) { a = dw_add(a, v); });
  double acc[1] = {dw_to_double_int(a)};
  grid_sum_finish<1>(acc, R, slot);
}

// slot <- sum of x (FP64 values): each thread sums its elements in
// double-word on the FP32 pipes (each value to 48 bits, the sum to about
// 2u^2 of the partial sums), the threads' sums are added in FP64
__global__ void __launch_bounds__(kRedThreads) k_sum_dw(const double* __restrict__ x, size_t n,
                                                        ReduceScratch R, int slot) {
  dw a{0.f, 0.f};
  stride4(n, [&](size_t q) { return x[q]; },
          [&](size_t, double v) { a = dw_add(a, dw_from_double_int(v)); });
  double acc[1] = {dw_to_double_int(a)};
  grid_sum_finish<1>(acc, R, slot);
}

// out = p - result[slot]/n: the difference in double-word (error about
// 2u^2 (|p| + |m|)), then converted exactly and summed in FP64 (one FP64
// addition per element)
__global__ void k_dw_out(const float2* __restrict__ p, double* __restrict__ out, size_t n,
                         ReduceScratch R, int slot) {
  const double m = R.result[slot] / (double)n;
  const dw mneg = dw_neg(dw_from_double(m));
  stride4(n, [&](size_t q) { return dw_ldg(p + q); },
          [&](size_t q, dw v) { out[q] = dw_to_double_int(dw_add(v, mneg)); });
}

// out += double(d): the correction of a warm-started solve added to its start
__global__ void k_dw_accumulate(const float2* __restrict__ d, double* __restrict__ out, size_t n) {
  stride4(n, [&](size_t q) { return dw_ldg(d + q); },
          [&](size_t q, dw v) { out[q] += dw_to_double_int(v); });
}

// The right-hand side's preparation in one pass: b -= m (m = result[mslot]/n;
// mslot < 0: no shift, b not written), sum (b - m)^2 -> result[slot2] (the
// order of k_shift_by_mean / k_sum, so the same bits), and, when given, the
// double-word copy bw and b rounded to float into r32 (the mixed solve's
// first residual for p = 0), colour-split when hstride != 0.
// The colour (i + j + k) & 1 of the cells a grid-stride loop visits, kept
// up to date by additions (integer division runs its conversions on GB300's
// FP64 pipe): set at the thread's first cell, advanced by the stride.
struct ColourWalk {
  int i, j, kp;     // x, y and the parity of z of the current cell
  int si, sj, skp;  // the stride split the same way
  int nx, ny;
  __device__ ColourWalk(size_t q, size_t s, int nx_, int ny_) : nx(nx_), ny(ny_) {
    const size_t row = q / (size_t)nx, srow = s / (size_t)nx;
    i = (int)(q - row * nx);
    j = (int)(row % (size_t)ny);
    kp = (int)((row / (size_t)ny) & 1);
    si = (int)(s - srow * nx);
    sj = (int)(srow % (size_t)ny);
    skp = (int)((srow / (size_t)ny) & 1);
  }
  __device__ __forceinline__ int colour() const { return (i + j + kp) & 1; }
  __device__ __forceinline__ void advance() {
    i += si;
    int carry = i >= nx;
    if (carry) i -= nx;
    j += sj + carry;
    carry = j >= ny;
    if (carry) j -= ny;
    kp = (kp + skp + carry) & 1;
  }
};

// (a call, so that the FP64 fused multiply-add is not if-converted and
// issued for every element)
__device__ __noinline__ double add_square_rare(double acc, double a) { return acc + a * a; }

__global__ void __launch_bounds__(kRedThreads) k_rhs_prep(double* __restrict__ b, size_t n,
                                                          ReduceScratch R, int mslot, int slot2,
                                                          float2* __restrict__ bw,
                                                          float* __restrict__ r32, int nx, int ny,
                                                          size_t hstride) {
  const double m = mslot >= 0 ? R.result[mslot] / (double)n : 0.0;
  const size_t q0 = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  ColourWalk cw(q0, (size_t)gridDim.x * blockDim.x, nx, ny);
  // |b - m|^2 (it only sets the scale of the relative tolerance) summed per
  // thread in double-word on the FP32 pipes: a^2 = hi^2 + 2 hi lo to about
  // 2^-47; the shift itself is the one FP64 operation per element
  // (values outside 2^-60 <= |a| <= 2^60, whose squares would leave the
  // float range, go to an FP64 sum instead)
  dw sq{0.f, 0.f};
  double sq64 = 0.0;
  // stride4 calls use() for q0, q0 + s, q0 + 2s, ... in this order
  stride4(n, [&](size_t q) { return b[q]; }, [&](size_t q, double x) {
    const double a = mslot >= 0 ? x - m : x;
    if (mslot >= 0) b[q] = a;
    const dw v = dw_from_double_int(a);
    const float ah = fabsf(v.hi);
    if (ah == 0.f || (ah >= 0x1p-60f && ah <= 0x1p60f)) {
      const float p = v.hi * v.hi;
      float e = __fmaf_rn(v.hi, v.hi, -p);
      e = __fmaf_rn(2.f * v.hi, v.lo, e);
      sq = dw_add(sq, dw{p, e});
    } else {
      sq64 = add_square_rare(sq64, a);
    }
    if (bw) {
      bw[q] = make_float2(v.hi, v.lo);
      // v.hi is a rounded to nearest float
      if (r32) r32[hstride == 0 ? q : (size_t)cw.colour() * hstride + (q >> 1)] = v.hi;
      cw.advance();
    }
  });
  double acc[1] = {dw_to_double_int(sq) + sq64};
  grid_sum_finish<1>(acc, R, slot2);
}

inline unsigned stride_blocks(size_t n) {
  const size_t b = (n + kRedThreads - 1) / kRedThreads;
  return (unsigned)std::max<size_t>(1, std::min<size_t>(b, 152 * 8));
}

}  // namespace

void launch_rhs_prep(cudaStream_t s, double* b, size_t n, const ReduceScratch& R, int mslot,
                     int slot2, float2* bw, float* r32, int nx, int ny, size_t hstride) {
  const unsigned blocks = std::min<unsigned>(stride_blocks(n), (unsigned)R.max_blocks);
  k_rhs_prep<<<blocks, kRedThreads, 0, s>>>(b, n, R, mslot, slot2, bw, r32, nx, ny, hstride);
}

dim3 defect_grid(int nx, int ny, int nz) {
  return dim3((unsigned)((nx + kDTX - 1) / kDTX), (unsigned)((ny + kDTY - 1) / kDTY),
              (unsigned)((nz + kDZ - 1) / kDZ));
}

void launch_defect(cudaStream_t s, const DwOperator& A, const float2* pin, float2* pout,
                   const float* e, float* r32, const ReduceScratch& R, int slot, size_t hstride) {
  launch_pdl(k_defect, defect_grid(A.nx, A.ny, A.nz), dim3(kDTX, kDTY), 0, s, A, pin, pout, e,
             r32, R, slot, hstride);
}

// A 3D tiled map over a dense (nx, ny, nz) array (cuTensorMapEncodeTiled via
// the runtime's driver entry point, so the library links no libcuda).
bool make_tensor_map_3d(CUtensorMap* map, const void* base, CUtensorMapDataType type, int elem,
                        int nx, int ny, int nz, int bx, int by) {
  static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
  if (!encode) {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault,
                                         &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !fn)
      return false;
    encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  }
  if (((size_t)nx * elem) % 16 != 0 || ((size_t)bx * elem) % 16 != 0) return false;
  const cuuint64_t dims[3] = {(cuuint64_t)nx, (cuuint64_t)ny, (cuuint64_t)nz};
  const cuuint64_t strides[2] = {(cuuint64_t)nx * elem, (cuuint64_t)nx * ny * elem};
  const cuuint32_t box[3] = {(cuuint32_t)bx, (cuuint32_t)by, 1};
  const cuuint32_t estride[3] = {1, 1, 1};
  return encode(map, type, 3, const_cast<void*>(base), dims, strides, box, estride,
                CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

bool make_defect_maps(DefectMaps* m, const float2* p, const float* e, const float2* b,
                      const float2* cx, const float2* cy, const float2* cz, int nx, int ny,
                      int nz, size_t split_hstride) {
  const CUtensorMapDataType f32 = CU_TENSOR_MAP_DATA_TYPE_FLOAT32;
  const int nx2 = 2 * nx, bx2 = 2 * kQBX;
  bool ok = make_tensor_map_3d(&m->p, p, f32, 4, nx2, ny, nz, bx2, kQBY) &&
            make_tensor_map_3d(&m->b, b, f32, 4, nx2, ny, nz, bx2, kQBY) &&
            make_tensor_map_3d(&m->cx, cx, f32, 4, nx2, ny, nz, bx2, kQBY) &&
            make_tensor_map_3d(&m->cy, cy, f32, 4, nx2, ny, nz, bx2, kQBY) &&
            make_tensor_map_3d(&m->cz, cz, f32, 4, nx2, ny, nz, bx2, kQBY);
  if (e && split_hstride) {
    ok = ok && make_tensor_map_3d(&m->e, e, f32, 4, nx / 2, ny, nz, kQSEX, kQBY) &&
         make_tensor_map_3d(&m->e1, e + split_hstride, f32, 4, nx / 2, ny, nz, kQSEX, kQBY);
  } else if (e) {
    ok = ok && make_tensor_map_3d(&m->e, e, f32, 4, nx, ny, nz, kQEX, kQBY);
    m->e1 = m->e;
  } else {
    m->e = m->p;
    m->e1 = m->p;
  }
  return ok;
}

int defect_tma_init() {
  return cudaFuncSetAttribute(k_defect_tma, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)kQSmem) == cudaSuccess
             ? 0
             : -1;
}

void launch_defect_tma(cudaStream_t s, const DefectMaps& maps, int nx, int ny, int nz, bool use_e,
                       float2* pout, float* r32, const ReduceScratch& R, int slot, int* err,
                       size_t hstride) {
  launch_pdl(k_defect_tma, defect_grid(nx, ny, nz), dim3(kDTX, kDTY), kQSmem, s, maps, nx, ny, nz,
             use_e ? 1 : 0, pout, r32, R, slot, err, hstride);
}

void launch_to_dw(cudaStream_t s, const double* a, float2* out, size_t n) {
  k_to_dw<<<stride_blocks(n) * 2, kRedThreads, 0, s>>>(a, out, n);
}

void launch_sum_dw(cudaStream_t s, const double* x, size_t n, const ReduceScratch& R, int slot) {
  const unsigned b = std::min<unsigned>(stride_blocks(n), (unsigned)R.max_blocks);
  k_sum_dw<<<b, kRedThreads, 0, s>>>(x, n, R, slot);
}

void launch_dw_sum(cudaStream_t s, const float2* p, size_t n, const ReduceScratch& R, int slot) {
  const unsigned b = std::min<unsigned>(stride_blocks(n), (unsigned)R.max_blocks);
  k_dw_sum<<<b, kRedThreads, 0, s>>>(p, n, R, slot);
}

void launch_dw_out(cudaStream_t s, const float2* p, double* out, size_t n, const ReduceScratch& R,
                   int slot) {
  k_dw_out<<<stride_blocks(n) * 2, kRedThreads, 0, s>>>(p, out, n, R, slot);
}

void launch_dw_accumulate(cudaStream_t s, const float2* d, double* out, size_t n) {
  k_dw_accumulate<<<stride_blocks(n) * 2, kRedThreads, 0, s>>>(d, out, n);
}

}  // namespace gbmg
