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

// Copy rows [j_lo, j_hi) of plane k of one colour half into shared memory at
// dst + (j_lo - j_base) * hx (one bulk copy; completion counted on bar).
__device__ __forceinline__ uint32_t stage_rows(float* dst, const float* half, const SweepArgs& A,
                                               int k, int j_base, int j_lo, int j_hi,
                                               uint64_t* bar) {
  j_lo = max(j_lo, 0);
  j_hi = min(j_hi, A.ny);
  if (j_hi <= j_lo) return 0;
  const uint32_t bytes = (uint32_t)(j_hi - j_lo) * (uint32_t)A.hx * 4u;
  const float* src = half + ((size_t)k * A.ny + j_lo) * A.hx;
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
      ::"r"(smem_u32(dst + (size_t)(j_lo - j_base) * A.hx)), "l"(src), "r"(bytes),
      "r"(smem_u32(bar))
      : "memory");
  return bytes;
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

// kZero: the first colour relaxes from p = 0 (the first sweep after a zero
// initial guess), so p_in is not read at all.
template <bool kZero>
__global__ void __launch_bounds__(384) k_sweep_split(SweepArgs A) {
  pdl_enter();
  extern __shared__ unsigned char sw_raw[];
  float* sm = reinterpret_cast<float*>((reinterpret_cast<uintptr_t>(sw_raw) + 127) &
                                       ~uintptr_t(127));
  uint64_t* bar = reinterpret_cast<uint64_t*>(sm + (size_t)A.o_new + (size_t)kSwNew * (A.by + 2) * A.hx);
  const int tq = A.hx >> 2;                 // threads per row
  const int q = threadIdx.x % tq, ra = threadIdx.x / tq;  // ra: row 0 .. by+1 (j0-1 .. j0+by)
  const int m0 = 4 * q;
  const int rg = blockIdx.x % A.nrg, ch = blockIdx.x / A.nrg;
  const int j0 = rg * A.by;
  const int z0 = ch * A.zc, z1 = min(A.nz, z0 + A.zc);
  const int jj = j0 - 1 + ra;
  const bool row_in = jj >= 0 && jj < A.ny;
  const int c1 = 1 - A.c0;
  const size_t sz = (size_t)A.hx * A.ny;
  const float* pB_g = A.pin + (size_t)c1 * A.hstride;
  const float* rB_g = A.rho + (size_t)c1 * A.hstride;
  const float* rA_g = A.rho + (size_t)A.c0 * A.hstride;
  const float* bA_g = A.src + (size_t)A.c0 * A.hstride;
  const float* bB_g = A.src + (size_t)c1 * A.hstride;
  float* pA_o = A.pout + (size_t)A.c0 * A.hstride;
  float* pB_o = A.pout + (size_t)c1 * A.hstride;
  // planes staged: [qlo, qhi]
  const int qlo = max(0, z0 - 2), qhi = min(A.nz - 1, z1 + 1);
  const int rowsB = A.by + 4, rowsA = A.by + 2;
  const auto slot_of = [&](int k) { return (k - qlo) % kSwStages; };
  const auto stage_pB = [&](int k) { return sm + (size_t)slot_of(k) * A.stage; };
  const auto stage_rB = [&](int k) { return sm + (size_t)slot_of(k) * A.stage + A.o_rB; };
  const auto stage_rA = [&](int k) { return sm + (size_t)slot_of(k) * A.stage + A.o_rA; };
  const auto new_row = [&](int k, int r) {
    return sm + A.o_new + ((size_t)(k % kSwNew) * rowsA + r) * A.hx;
  };
  if (threadIdx.x == 0) {
    for (int s = 0; s < kSwStages; ++s) mbar_init(&bar[s], 1);
    fence_barrier_init();
  }
  __syncthreads();
  const auto issue = [&](int k) {  // one thread
    const int s = slot_of(k);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    // expected bytes first, then the copies
    uint32_t bytes = 0;
    const int lo = max(j0 - 2, 0), hi = min(j0 + A.by + 2, A.ny);
    const int loA = max(j0 - 1, 0), hiA = min(j0 + A.by + 1, A.ny);
    bytes += (uint32_t)(hi - lo) * A.hx * 4u * (kZero ? 1u : 2u);
    bytes += (uint32_t)(hiA - loA) * A.hx * 4u;
    mbar_arrive_expect_tx(&bar[s], bytes);
    if (!kZero) stage_rows(stage_pB(k), pB_g, A, k, j0 - 2, j0 - 2, j0 + A.by + 2, &bar[s]);
    stage_rows(stage_rB(k), rB_g, A, k, j0 - 2, j0 - 2, j0 + A.by + 2, &bar[s]);
    stage_rows(stage_rA(k), rA_g, A, k, j0 - 1, j0 - 1, j0 + A.by + 1, &bar[s]);
  };
  int issued = qlo - 1, waited = qlo - 1;
  const int t0 = max(z0 - 1, 0);
  if (threadIdx.x == 0)
    for (int k = qlo; k <= min(qhi, t0 + 2); ++k) issue(k);
  issued = min(qhi, t0 + 2);
  const float inf = __int_as_float(0x7f800000);
  for (int t = t0; t <= z1; ++t) {
    if (t + 2 <= qhi && t + 2 > issued) {
      if (threadIdx.x == 0) issue(t + 2);
      issued = t + 2;
    }
    // this step's right-hand sides straight into registers
    const bool doA = row_in && t < A.nz;
    const int u = t - 1;
    const bool doB = row_in && ra >= 1 && ra <= A.by && u >= z0 && u < z1;
    float bA[4] = {0.f, 0.f, 0.f, 0.f}, bB[4] = {0.f, 0.f, 0.f, 0.f};
    if (doA) unpack4(__ldg(reinterpret_cast<const float4*>(bA_g + t * sz + (size_t)jj * A.hx + m0)), bA);
    if (doB) unpack4(__ldg(reinterpret_cast<const float4*>(bB_g + u * sz + (size_t)jj * A.hx + m0)), bB);
    const int need = min(t + 1, qhi);
    while (waited < need) {
      ++waited;
      const int s = slot_of(waited);
      mbar_wait(&bar[s], (uint32_t)(((waited - qlo) / kSwStages) & 1), A.err);
    }
    // colour A of plane t on rows j0-1 .. j0+by
    if (doA) {
      const int par = (jj + t + A.c0) & 1;
      const int rb_ = ra + 1;  // row jj in the by+4 row arrays
      const float* rB = stage_rB(t);
      const float* pB = stage_pB(t);
      float rc[4];
      unpack4(lds4(stage_rA(t) + (size_t)ra * A.hx + m0), rc);
      float rxm[4], rxp[4], pxm[4], pxp[4];
      x_window(rB + (size_t)rb_ * A.hx, pB + (size_t)rb_ * A.hx, m0, A.hx, par, kZero, rxm, rxp,
               pxm, pxp);
      float rym[4], pym[4], ryp[4], pyp[4], rzm[4], pzm[4], rzp[4], pzp[4];
      nb_row(rB + (size_t)(rb_ - 1) * A.hx, pB + (size_t)(rb_ - 1) * A.hx, m0, jj > 0, kZero,
             rym, pym);
      nb_row(rB + (size_t)(rb_ + 1) * A.hx, pB + (size_t)(rb_ + 1) * A.hx, m0, jj < A.ny - 1,
             kZero, ryp, pyp);
      if (t > 0)
        nb_row(stage_rB(t - 1) + (size_t)rb_ * A.hx, stage_pB(t - 1) + (size_t)rb_ * A.hx, m0,
               true, kZero, rzm, pzm);
      else
        nb_row(rB, pB, m0, false, kZero, rzm, pzm);
      if (t < A.nz - 1)
        nb_row(stage_rB(t + 1) + (size_t)rb_ * A.hx, stage_pB(t + 1) + (size_t)rb_ * A.hx, m0,
               true, kZero, rzp, pzp);
      else
        nb_row(rB, pB, m0, false, kZero, rzp, pzp);
      const float4 v = relax4<kZero>(A, rc, bA, rxm, rxp, pxm, pxp, rym, pym, ryp, pyp, rzm, pzm,
                                     rzp, pzp);
      sts4(new_row(t, ra) + m0, v);
      if (ra >= 1 && ra <= A.by && t >= z0 && t < z1)
        *reinterpret_cast<float4*>(pA_o + t * sz + (size_t)jj * A.hx + m0) = v;
    }
    __syncthreads();
    // colour B of plane u = t-1 on the block's rows, from the new colour A
    if (doB) {
      const int par = (jj + u + c1) & 1;
      float rc[4];
      unpack4(lds4(stage_rB(u) + (size_t)(ra + 1) * A.hx + m0), rc);
      const float* rA = stage_rA(u);
      float rxm[4], rxp[4], pxm[4], pxp[4];
      x_window(rA + (size_t)ra * A.hx, new_row(u, ra), m0, A.hx, par, false, rxm, rxp, pxm, pxp);
      float rym[4], pym[4], ryp[4], pyp[4], rzm[4], pzm[4], rzp[4], pzp[4];
      nb_row(rA + (size_t)(ra - 1) * A.hx, new_row(u, ra - 1), m0, jj > 0, false, rym, pym);
      nb_row(rA + (size_t)(ra + 1) * A.hx, new_row(u, ra + 1), m0, jj < A.ny - 1, false, ryp, pyp);
      if (u > 0)
        nb_row(stage_rA(u - 1) + (size_t)ra * A.hx, new_row(u - 1, ra), m0, true, false, rzm, pzm);
      else
        nb_row(rA, rA, m0, false, false, rzm, pzm);
      if (u < A.nz - 1)
        nb_row(stage_rA(u + 1) + (size_t)ra * A.hx, new_row(u + 1, ra), m0, true, false, rzp, pzp);
      else
        nb_row(rA, rA, m0, false, false, rzp, pzp);
      const float4 v = relax4<false>(A, rc, bB, rxm, rxp, pxm, pxp, rym, pym, ryp, pyp, rzm, pzm,
                                     rzp, pzp);
      *reinterpret_cast<float4*>(pB_o + u * sz + (size_t)jj * A.hx + m0) = v;
    }
    __syncthreads();
  }
  (void)inf;
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
  S.smem = (int)(floats * sizeof(float) + kSwStages * sizeof(uint64_t) + 128);
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
