// One whole red-black Gauss-Seidel sweep of the colour-split FP32 finest
// level per launch (sm_103a).
//
// The two-launch sweep (k_smooth_split4 once per colour) moves about 18-20
// bytes per cell: the second launch re-reads the density and the first
// colour's pressure after the first launch has evicted part of them from L2.
// This kernel does both colours in one pass over z, out of place (p_in ->
// p_out): at step t it relaxes the first colour (A) of plane t from p_in's
// second colour (B), then colour B of plane t-1 from the new colour A of
// planes t-2 .. t.  Colour B of p_in is the only part of p_in it reads
// (colour A's old values are never needed by a Gauss-Seidel update), so one
// sweep moves
//     p_in colour B (2 B/cell) + b (4) + rho (4) in, p_out (4) out = 14 B/cell.
//
// Blocks own `by` whole rows of a chunk of z planes.  Each plane's rows of p_in
// colour B and rho colour B (by + 4 rows: the rows of colour A's y neighbours)
// and rho colour A (by + 2 rows) stream into a 5-stage shared-memory ring by
// cp.async.bulk (one contiguous copy per array: a plane's rows of one colour
// half are contiguous), two planes ahead of the compute, with an mbarrier per
// stage; b is read straight into registers.  Colour A is also relaxed on the
// row above and the row below the block and on the plane under the chunk, so
// that colour B needs no other block's values; the block stores only its own
// rows and planes.  Every block reads the same p_in and writes only its own
// cells of p_out, so the result does not depend on the schedule, and it equals
// the two-launch sweep bit for bit: each cell's update is the same sequence of
// pinned roundings (rho_face32, rho_acc32, rho_relax32) over the faces in the
// order x-, x+, y-, y+, z-, z+, with wall neighbours at density +inf and
// pressure 0 as there.
//
// Smoother of the reference's cycle: multigrid_relax
// ("DomainDecomposition/3D/src/others/multigrid_solver.f90:1-49") with the
// variable-coefficient update of ppe_sor_solver ("Two phase flows/newOpenMP/
// 3D+IBM/src/ns_solver/ns_ppe_solver.f90:97-115").
#include <algorithm>

#include "gbmg_internal.h"
#include "pdl.cuh"
#include "tma.cuh"

namespace gbmg {

namespace {

constexpr int kSwStages = 5;  // plane stages of the ring
constexpr int kSwNew = 3;     // planes of new colour-A values kept

struct SweepArgs {
  const float* rho;  // colour-split density, pressure and right-hand side
  const float* src;
  const float* pin;
  float* pout;
  size_t hstride;
  int nx, ny, nz, hx;
  int by;   // rows stored per block
  int zc;   // z planes per block
  int nrg;  // row groups
  float kx, ky, kz;
  int c0;   // first colour
  int* err;
  // shared memory (floats): per stage pB (by+4 rows), rB (by+4), rA (by+2);
  // then the new colour-A ring (kSwNew planes of by+2 rows)
  int stage, o_rB, o_rA, o_new;
};

__device__ __forceinline__ float4 lds4(const float* p) {
  return *reinterpret_cast<const float4*>(p);
}
__device__ __forceinline__ void sts4(float* p, float4 v) { *reinterpret_cast<float4*>(p) = v; }
__device__ __forceinline__ void unpack4(float4 v, float (&a)[4]) {
  a[0] = v.x; a[1] = v.y; a[2] = v.z; a[3] = v.w;
}

// The x window of a cell quad m0..m0+3 of colour parity `par` in a row of the
// other colour: x- neighbours at half index m-1+par, x+ at m+par (walls: +inf
// density, zero pressure), as k_smooth_split4 forms them.
__device__ __forceinline__ void x_window(const float* row_r, const float* row_p, int m0, int hx,
                                         int par, bool zero, float (&rxm)[4], float (&rxp)[4],
                                         float (&pxm)[4], float (&pxp)[4]) {
  const float inf = __int_as_float(0x7f800000);
  float rv[4], pv[4] = {0.f, 0.f, 0.f, 0.f};
  unpack4(lds4(row_r + m0), rv);
  if (!zero) unpack4(lds4(row_p + m0), pv);
  float re = inf, pe = 0.f;
  if (par) {
    if (m0 + 4 < hx) { re = row_r[m0 + 4]; if (!zero) pe = row_p[m0 + 4]; }
    rxm[0] = rv[0]; rxm[1] = rv[1]; rxm[2] = rv[2]; rxm[3] = rv[3];
    rxp[0] = rv[1]; rxp[1] = rv[2]; rxp[2] = rv[3]; rxp[3] = re;
    pxm[0] = pv[0]; pxm[1] = pv[1]; pxm[2] = pv[2]; pxm[3] = pv[3];
    pxp[0] = pv[1]; pxp[1] = pv[2]; pxp[2] = pv[3]; pxp[3] = pe;
  } else {
    if (m0 > 0) { re = row_r[m0 - 1]; if (!zero) pe = row_p[m0 - 1]; }
    rxm[0] = re; rxm[1] = rv[0]; rxm[2] = rv[1]; rxm[3] = rv[2];
    rxp[0] = rv[0]; rxp[1] = rv[1]; rxp[2] = rv[2]; rxp[3] = rv[3];
    pxm[0] = pe; pxm[1] = pv[0]; pxm[2] = pv[1]; pxm[3] = pv[2];
    pxp[0] = pv[0]; pxp[1] = pv[1]; pxp[2] = pv[2]; pxp[3] = pv[3];
  }
}

// A neighbour row (y or z) of the other colour, or a wall.
__device__ __forceinline__ void nb_row(const float* row_r, const float* row_p, int m0, bool valid,
                                       bool zero, float (&r)[4], float (&p)[4]) {
  const float inf = __int_as_float(0x7f800000);
  if (valid) {
    unpack4(lds4(row_r + m0), r);
    if (!zero) unpack4(lds4(row_p + m0), p);
    else p[0] = p[1] = p[2] = p[3] = 0.f;
  } else {
    r[0] = r[1] = r[2] = r[3] = inf;
    p[0] = p[1] = p[2] = p[3] = 0.f;
  }
}

// The four cells' updates from their six neighbours (k_smooth_split4's
// arithmetic, face order x-, x+, y-, y+, z-, z+).
template <bool kZero>
__device__ __forceinline__ float4 relax4(const SweepArgs& A, const float (&rc)[4],
                                         const float (&b)[4], const float (&rxm)[4],
                                         const float (&rxp)[4], const float (&pxm)[4],
                                         const float (&pxp)[4], const float (&rym)[4],
                                         const float (&pym)[4], const float (&ryp)[4],
                                         const float (&pyp)[4], const float (&rzm)[4],
                                         const float (&pzm)[4], const float (&rzp)[4],
                                         const float (&pzp)[4]) {
  float out[4];
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    float s = 0.f, d = 0.f, cc;
    cc = rho_face32(A.kx, rc[c], rxm[c]); if (!kZero) rho_acc32(cc, pxm[c], s, d); else d = __fadd_rn(d, cc);
    cc = rho_face32(A.kx, rc[c], rxp[c]); if (!kZero) rho_acc32(cc, pxp[c], s, d); else d = __fadd_rn(d, cc);
    cc = rho_face32(A.ky, rc[c], rym[c]); if (!kZero) rho_acc32(cc, pym[c], s, d); else d = __fadd_rn(d, cc);
    cc = rho_face32(A.ky, rc[c], ryp[c]); if (!kZero) rho_acc32(cc, pyp[c], s, d); else d = __fadd_rn(d, cc);
    cc = rho_face32(A.kz, rc[c], rzm[c]); if (!kZero) rho_acc32(cc, pzm[c], s, d); else d = __fadd_rn(d, cc);
    cc = rho_face32(A.kz, rc[c], rzp[c]); if (!kZero) rho_acc32(cc, pzp[c], s, d); else d = __fadd_rn(d, cc);
    out[c] = rho_relax32(s, b[c], d);
  }
  return make_float4(out[0], out[1], out[2], out[3]);
}

// Pointers to one plane's staged rows of each array, and to its new colour-A
// rows, offset to this thread's quad.
struct PlaneRows {
  const float* pB;  // row jj of p_in colour B (by+4-row array)
  const float* rB;  // row jj of rho colour B
  const float* rA;  // row jj of rho colour A (by+2-row array)
  float* nA;        // row jj of the new colour A
};

// kZero: the first colour relaxes from p = 0 (the first sweep after a zero
// initial guess), so p_in is not read at all.
template <bool kZero>
__global__ void __launch_bounds__(384) k_sweep_split(SweepArgs A) {
  pdl_enter();
  extern __shared__ float4 sw_smem[];
  float* const sm = reinterpret_cast<float*>(sw_smem);
  const int hx = A.hx;
  const int rowsA = A.by + 2;
  uint64_t* bar = reinterpret_cast<uint64_t*>(sm + A.o_new + kSwNew * rowsA * hx);
  const int tq = hx >> 2;                                 // threads per row
  const int q = threadIdx.x % tq, ra = threadIdx.x / tq;  // ra: row j0-1 .. j0+by
  const int m0 = 4 * q;
  const int rg = blockIdx.x % A.nrg, ch = blockIdx.x / A.nrg;
  const int j0 = rg * A.by;
  const int z0 = ch * A.zc, z1 = min(A.nz, z0 + A.zc);
  const int jj = j0 - 1 + ra;
  const bool row_in = jj >= 0 && jj < A.ny;
  const bool own_row = row_in && ra >= 1 && ra <= A.by;
  const bool ym_ok = jj > 0, yp_ok = jj < A.ny - 1;
  const int c1 = 1 - A.c0;
  const size_t sz = (size_t)hx * A.ny;
  const int offB = (ra + 1) * hx + m0;  // this thread's row in the by+4-row arrays
  const int offA = ra * hx + m0;        // ... and in the by+2-row arrays
  // planes staged: [qlo, qhi]
  const int qlo = max(0, z0 - 2), qhi = min(A.nz - 1, z1 + 1);
  const auto stage_base = [&](int slot) { return sm + slot * A.stage; };
  if (threadIdx.x == 0) {
    for (int s = 0; s < kSwStages; ++s) mbar_init(&bar[s], 1);
    fence_barrier_init();
  }
  __syncthreads();
  // the block's row ranges of the staged arrays, clamped to the grid
  const int loB = max(j0 - 2, 0), hiB = min(j0 + A.by + 2, A.ny);
  const int loA = max(j0 - 1, 0), hiA = min(j0 + A.by + 1, A.ny);
  const uint32_t bytesB = (uint32_t)(hiB - loB) * hx * 4u, bytesA = (uint32_t)(hiA - loA) * hx * 4u;
  const float* pB_g = A.pin + (size_t)c1 * A.hstride + (size_t)loB * hx;
  const float* rB_g = A.rho + (size_t)c1 * A.hstride + (size_t)loB * hx;
  const float* rA_g = A.rho + (size_t)A.c0 * A.hstride + (size_t)loA * hx;
  const int dstB = (loB - (j0 - 2)) * hx, dstA = (loA - (j0 - 1)) * hx;
  const auto issue = [&](int k) {  // one thread
    const int slot = (k - qlo) % kSwStages;
    float* base = stage_base(slot);
    uint64_t* b = &bar[slot];
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    mbar_arrive_expect_tx(b, (kZero ? 1u : 2u) * bytesB + bytesA);
    const size_t pk = (size_t)k * sz;
    const auto copy = [&](float* dst, const float* src, uint32_t bytes) {
      asm volatile(
          "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
          ::"r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(b))
          : "memory");
    };
    if (!kZero) copy(base + dstB, pB_g + pk, bytesB);
    copy(base + A.o_rB + dstB, rB_g + pk, bytesB);
    copy(base + A.o_rA + dstA, rA_g + pk, bytesA);
  };
  const int t0 = max(z0 - 1, 0);
  int issued = min(qhi, t0 + 2);
  if (threadIdx.x == 0)
    for (int k = qlo; k <= issued; ++k) issue(k);
  int waited = qlo - 1;
  // this thread's right-hand sides and outputs, advanced one plane per step
  // (offsets in signed arithmetic: plane t0 - 1 may be -1, never dereferenced)
  const ptrdiff_t off0 = (ptrdiff_t)t0 * (ptrdiff_t)sz + (ptrdiff_t)jj * hx + m0;
  const float* bA_p = A.src + (ptrdiff_t)A.c0 * (ptrdiff_t)A.hstride + off0;
  const float* bB_p = A.src + (ptrdiff_t)c1 * (ptrdiff_t)A.hstride + off0 - (ptrdiff_t)sz;
  float* oA_p = A.pout + (ptrdiff_t)A.c0 * (ptrdiff_t)A.hstride + off0;
  float* oB_p = A.pout + (ptrdiff_t)c1 * (ptrdiff_t)A.hstride + off0 - (ptrdiff_t)sz;
  // ring positions of planes t-2 .. t+1 (stages) and t-2 .. t (new colour A)
  int sl = (t0 - qlo) % kSwStages;  // slot of plane t
  int nl = t0 % kSwNew;             // new-ring slot of plane t
  const auto wrap5 = [](int v) { return v >= kSwStages ? v - kSwStages : (v < 0 ? v + kSwStages : v); };
  const auto wrap3 = [](int v) { return v >= kSwNew ? v - kSwNew : (v < 0 ? v + kSwNew : v); };
  const auto rows_of = [&](int slot, int nslot) {
    const float* base = stage_base(slot);
    return PlaneRows{base + offB, base + A.o_rB + offB, base + A.o_rA + offA,
                     sm + A.o_new + nslot * rowsA * hx + offA};
  };
  const int rowB = hx, rowA = hx;  // row pitch of the staged arrays
  for (int t = t0; t <= z1; ++t) {
    if (t + 2 <= qhi && t + 2 > issued) {
      if (threadIdx.x == 0) issue(t + 2);
      issued = t + 2;
    }
    const int u = t - 1;
    const bool doA = row_in && t < A.nz;
    const bool doB = own_row && u >= z0 && u < z1;
    float bA[4] = {0.f, 0.f, 0.f, 0.f}, bB[4] = {0.f, 0.f, 0.f, 0.f};
    if (doA) unpack4(__ldg(reinterpret_cast<const float4*>(bA_p)), bA);
    if (doB) unpack4(__ldg(reinterpret_cast<const float4*>(bB_p)), bB);
    const int need = min(t + 1, qhi);
    while (waited < need) {
      ++waited;
      const int slot = (waited - qlo) % kSwStages;
      mbar_wait(&bar[slot], (uint32_t)(((waited - qlo) / kSwStages) & 1), A.err);
    }
    const PlaneRows Pm = rows_of(wrap5(sl - 1), wrap3(nl - 1));  // plane t-1
    const PlaneRows P0 = rows_of(sl, nl);                          // plane t
    // colour A of plane t on rows j0-1 .. j0+by
    if (doA) {
      const PlaneRows Pp = rows_of(wrap5(sl + 1), nl);  // plane t+1 (stages only)
      const int par = (jj + t + A.c0) & 1;
      float rc[4];
      unpack4(lds4(P0.rA), rc);
      float rxm[4], rxp[4], pxm[4], pxp[4];
      x_window(P0.rB - m0, P0.pB - m0, m0, hx, par, kZero, rxm, rxp, pxm, pxp);
      float rym[4], pym[4], ryp[4], pyp[4], rzm[4], pzm[4], rzp[4], pzp[4];
      nb_row(P0.rB - rowB - m0, P0.pB - rowB - m0, m0, ym_ok, kZero, rym, pym);
      nb_row(P0.rB + rowB - m0, P0.pB + rowB - m0, m0, yp_ok, kZero, ryp, pyp);
      nb_row(Pm.rB - m0, Pm.pB - m0, m0, t > 0, kZero, rzm, pzm);
      nb_row(Pp.rB - m0, Pp.pB - m0, m0, t < A.nz - 1, kZero, rzp, pzp);
      const float4 v = relax4<kZero>(A, rc, bA, rxm, rxp, pxm, pxp, rym, pym, ryp, pyp, rzm, pzm,
                                     rzp, pzp);
      sts4(P0.nA, v);
      if (own_row && t >= z0 && t < z1) *reinterpret_cast<float4*>(oA_p) = v;
    }
    __syncthreads();
    // colour B of plane u = t-1 on the block's rows, from the new colour A
    if (doB) {
      const PlaneRows Pmm = rows_of(wrap5(sl - 2), wrap3(nl - 2));  // plane u-1
      const int par = (jj + u + c1) & 1;
      float rc[4];
      unpack4(lds4(Pm.rB), rc);
      float rxm[4], rxp[4], pxm[4], pxp[4];
      x_window(Pm.rA - m0, Pm.nA - m0, m0, hx, par, false, rxm, rxp, pxm, pxp);
      float rym[4], pym[4], ryp[4], pyp[4], rzm[4], pzm[4], rzp[4], pzp[4];
      nb_row(Pm.rA - rowA - m0, Pm.nA - rowA - m0, m0, ym_ok, false, rym, pym);
      nb_row(Pm.rA + rowA - m0, Pm.nA + rowA - m0, m0, yp_ok, false, ryp, pyp);
      nb_row(Pmm.rA - m0, Pmm.nA - m0, m0, u > 0, false, rzm, pzm);
      nb_row(P0.rA - m0, P0.nA - m0, m0, u < A.nz - 1, false, rzp, pzp);
      const float4 v = relax4<false>(A, rc, bB, rxm, rxp, pxm, pxp, rym, pym, ryp, pyp, rzm, pzm,
                                     rzp, pzp);
      *reinterpret_cast<float4*>(oB_p) = v;
    }
    __syncthreads();
    sl = wrap5(sl + 1);
    nl = wrap3(nl + 1);
    bA_p += sz;
    bB_p += sz;
    oA_p += sz;
    oB_p += sz;
  }
}

struct SweepShape {
  int by, threads, smem, stage, o_rB, o_rA, o_new;
};

// Rows per block for a row of hx half cells: about 256-384 threads.
SweepShape sweep_shape(int hx) {
  SweepShape S{};
  const int tq = hx / 4;
  S.by = hx <= 64 ? 16 : (hx <= 128 ? 8 : 4);
  S.threads = tq * (S.by + 2);
  S.stage = hx * (2 * (S.by + 4) + (S.by + 2));
  S.stage = (S.stage + 31) & ~31;  // 128-byte aligned stages
  S.o_rB = hx * (S.by + 4);
  S.o_rA = 2 * hx * (S.by + 4);
  S.o_new = kSwStages * S.stage;
  const size_t floats = (size_t)S.o_new + (size_t)kSwNew * (S.by + 2) * hx;
  S.smem = (int)(floats * sizeof(float) + kSwStages * sizeof(uint64_t));
  return S;
}

}  // namespace

bool sweep_split_supported(int nx, int ny, int nz, size_t hstride) {
  (void)ny;
  (void)nz;
  const int hx = nx / 2;
  if (nx % 8 != 0 || hx > 256 || hstride % 4 != 0) return false;
  const SweepShape S = sweep_shape(hx);
  return S.threads <= 384 && S.smem <= 227 * 1024;
}

// Both variants may use up to 227 KB of dynamic shared memory (each launch
// asks for what its row width needs).
int sweep_split_init() {
  constexpr int kMax = 227 * 1024;
  cudaError_t e = cudaFuncSetAttribute(k_sweep_split<false>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, kMax);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_sweep_split<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             kMax);
  if (e != cudaSuccess) cudaGetLastError();
  return e == cudaSuccess ? 0 : 1;
}

void launch_sweep_split(cudaStream_t s, const LevelView<float>& L, const float* pin, float* pout,
                        int first_color, bool zero_guess, int* err) {
  const int hx = L.nx / 2;
  const SweepShape S = sweep_shape(hx);
  SweepArgs A{};
  A.rho = L.rho;
  A.src = L.src;
  A.pin = pin;
  A.pout = pout;
  A.hstride = L.hstride;
  A.nx = L.nx; A.ny = L.ny; A.nz = L.nz; A.hx = hx;
  A.by = S.by;
  A.nrg = (L.ny + S.by - 1) / S.by;
  A.kx = L.kx; A.ky = L.ky; A.kz = L.kz;
  A.c0 = first_color;
  A.err = err;
  A.stage = S.stage; A.o_rB = S.o_rB; A.o_rA = S.o_rA; A.o_new = S.o_new;
  // z chunks: as many as fill the resident blocks of the device in one wave
  static int sms = 0;
  if (!sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 1;
  }
  int per_sm = 1;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_sweep_split<false>, S.threads, S.smem);
  per_sm = std::max(per_sm, 1);
  const int slots = sms * per_sm;
  const int nch = std::max(1, std::min(L.nz, slots / A.nrg));
  A.zc = (L.nz + nch - 1) / nch;
  const int chunks = (L.nz + A.zc - 1) / A.zc;
  const dim3 grid((unsigned)(A.nrg * chunks));
  if (zero_guess)
    launch_pdl(k_sweep_split<true>, grid, dim3(S.threads), (size_t)S.smem, s, A);
  else
    launch_pdl(k_sweep_split<false>, grid, dim3(S.threads), (size_t)S.smem, s, A);
}

}  // namespace gbmg
