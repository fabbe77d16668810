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
constexpr int kSwGuard = 4;   // guard floats before and after every staged row

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
  // shared memory (floats): rows of rp = hx + 2*kSwGuard floats (the row's
  // cells start at kSwGuard; the guards hold the wall values).  Per stage:
  // pB (by+4 rows), rB (by+4), rA (by+2); then the new colour-A ring (kSwNew
  // planes of by+2 rows), a wall density row (+inf) and a wall pressure row (0).
  int rp, stage, o_rB, o_rA, o_new, o_wall;
};

__device__ __forceinline__ float4 lds4(const float* p) {
  return *reinterpret_cast<const float4*>(p);
}
__device__ __forceinline__ void unpack4(float4 v, float (&a)[4]) {
  a[0] = v.x; a[1] = v.y; a[2] = v.z; a[3] = v.w;
}

// The x window of a cell quad m0..m0+3 of colour parity par in a row of the
// other colour: x- neighbours at half index m-1+par, x+ at m+par.  rowc points
// at the row's cell m0 - 1 + par; a wall is a guard value (+inf density, zero
// pressure), as k_smooth_split4 substitutes them.
__device__ __forceinline__ void x_window(const float* rowr, const float* rowp, bool zero,
                                         float (&rxm)[4], float (&rxp)[4], float (&pxm)[4],
                                         float (&pxp)[4]) {
  float w[5], v[5];
#pragma unroll
  for (int c = 0; c < 5; ++c) {
    w[c] = rowr[c];
    v[c] = zero ? 0.f : rowp[c];
  }
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    rxm[c] = w[c];
    rxp[c] = w[c + 1];
    pxm[c] = v[c];
    pxp[c] = v[c + 1];
  }
}

// A neighbour row (y or z) of the other colour (a wall row when outside).
__device__ __forceinline__ void nb_row(const float* rowr, const float* rowp, bool zero,
                                       float (&r)[4], float (&p)[4]) {
  unpack4(lds4(rowr), r);
  if (!zero) unpack4(lds4(rowp), p);
  else p[0] = p[1] = p[2] = p[3] = 0.f;
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
__global__ void __launch_bounds__(640, 1) k_sweep_split(SweepArgs A) {
  pdl_enter();
  extern __shared__ float4 sw_smem[];
  float* const sm = reinterpret_cast<float*>(sw_smem);
  const int hx = A.hx, rp = A.rp;
  const int rowsA = A.by + 2, rowsB = A.by + 4;
  uint64_t* bar = reinterpret_cast<uint64_t*>(sm + A.o_wall + 2 * rp);
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
  const float* wall_r = sm + A.o_wall + kSwGuard;       // +inf row
  const float* wall_p = sm + A.o_wall + rp + kSwGuard;  // zero row
  // guards and wall rows: +inf for densities, 0 for pressures, written once
  {
    const float inf = __int_as_float(0x7f800000);
    const int nrows = kSwStages * (2 * rowsB + rowsA) + kSwNew * rowsA;
    for (int e = threadIdx.x; e < nrows * 2 * kSwGuard; e += blockDim.x) {
      const int row = e / (2 * kSwGuard), g = e % (2 * kSwGuard);
      const int col = g < kSwGuard ? g : hx + g;  // 0..3 and hx+4..hx+7
      float* base;
      bool dens;
      if (row < kSwStages * (2 * rowsB + rowsA)) {
        const int st = row / (2 * rowsB + rowsA), r = row % (2 * rowsB + rowsA);
        base = sm + st * A.stage + r * rp;  // pB rows, then rB, then rA
        dens = r >= rowsB;
      } else {
        base = sm + A.o_new + (row - kSwStages * (2 * rowsB + rowsA)) * rp;
        dens = false;
      }
      base[col] = dens ? inf : 0.f;
    }
    for (int e = threadIdx.x; e < rp; e += blockDim.x) {
      sm[A.o_wall + e] = inf;
      sm[A.o_wall + rp + e] = 0.f;
    }
  }
  // planes staged: [qlo, qhi]
  const int qlo = max(0, z0 - 2), qhi = min(A.nz - 1, z1 + 1);
  if (threadIdx.x == 0) {
    for (int s = 0; s < kSwStages; ++s) mbar_init(&bar[s], 1);
    fence_barrier_init();
  }
  __syncthreads();
  // the block's row ranges of the staged arrays, clamped to the grid
  const int loB = max(j0 - 2, 0), hiB = min(j0 + A.by + 2, A.ny);
  const int loA = max(j0 - 1, 0), hiA = min(j0 + A.by + 1, A.ny);
  const int nB = hiB - loB, nA = hiA - loA;
  const uint32_t row_bytes = (uint32_t)hx * 4u;
  const float* pB_g = A.pin + (size_t)c1 * A.hstride + (size_t)loB * hx;
  const float* rB_g = A.rho + (size_t)c1 * A.hstride + (size_t)loB * hx;
  const float* rA_g = A.rho + (size_t)A.c0 * A.hstride + (size_t)loA * hx;
  const int dB = loB - (j0 - 2), dA = loA - (j0 - 1);  // first staged row's index
  // one plane's rows into its stage, a row per copy (rows are padded in shared
  // memory), issued by the lanes of warp 0
  const auto issue = [&](int k) {
    const int slot = (k - qlo) % kSwStages;
    float* base = sm + slot * A.stage;
    uint64_t* b = &bar[slot];
    const int lane = threadIdx.x;  // warp 0
    if (lane == 0) {
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      mbar_arrive_expect_tx(b, ((kZero ? 1u : 2u) * nB + nA) * row_bytes);
    }
    __syncwarp();
    const size_t pk = (size_t)k * sz;
    const int ncopy = (kZero ? 0 : nB) + nB + nA;
    for (int c = lane; c < ncopy; c += 32) {
      float* dst;
      const float* src;
      if (!kZero && c < nB) {
        dst = base + (dB + c) * rp + kSwGuard;
        src = pB_g + pk + (size_t)c * hx;
      } else {
        const int cc = kZero ? c : c - nB;
        if (cc < nB) {
          dst = base + A.o_rB + (dB + cc) * rp + kSwGuard;
          src = rB_g + pk + (size_t)cc * hx;
        } else {
          dst = base + A.o_rA + (dA + cc - nB) * rp + kSwGuard;
          src = rA_g + pk + (size_t)(cc - nB) * hx;
        }
      }
      asm volatile(
          "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
          ::"r"(smem_u32(dst)), "l"(src), "r"(row_bytes), "r"(smem_u32(b))
          : "memory");
    }
  };
  const int t0 = max(z0 - 1, 0);
  int issued = min(qhi, t0 + 2);
  if (threadIdx.x < 32)
    for (int k = qlo; k <= issued; ++k) issue(k);
  int waited = qlo - 1;
  // this thread's right-hand sides and outputs, advanced one plane per step
  // (signed offsets: plane t0 - 1 may be -1, never dereferenced)
  const ptrdiff_t off0 = (ptrdiff_t)t0 * (ptrdiff_t)sz + (ptrdiff_t)jj * hx + m0;
  const float* bA_p = A.src + (ptrdiff_t)A.c0 * (ptrdiff_t)A.hstride + off0;
  const float* bB_p = A.src + (ptrdiff_t)c1 * (ptrdiff_t)A.hstride + off0 - (ptrdiff_t)sz;
  float* oA_p = A.pout + (ptrdiff_t)A.c0 * (ptrdiff_t)A.hstride + off0;
  float* oB_p = A.pout + (ptrdiff_t)c1 * (ptrdiff_t)A.hstride + off0 - (ptrdiff_t)sz;
  // this thread's offsets inside a stage and the new ring (cell m0 of its row)
  const int offB = (ra + 1) * rp + kSwGuard + m0;
  const int offA = ra * rp + kSwGuard + m0;
  int sl = (t0 - qlo) % kSwStages;  // stage slot of plane t
  int nl = t0 % kSwNew;             // new-ring slot of plane t
  const auto wrap5 = [](int v) { return v >= kSwStages ? v - kSwStages : (v < 0 ? v + kSwStages : v); };
  const auto wrap3 = [](int v) { return v >= kSwNew ? v - kSwNew : (v < 0 ? v + kSwNew : v); };
  for (int t = t0; t <= z1; ++t) {
    if (t + 2 <= qhi && t + 2 > issued) {
      if (threadIdx.x < 32) issue(t + 2);
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
    const float* S0 = sm + sl * A.stage;
    const float* Sm = sm + wrap5(sl - 1) * A.stage;
    const float* Sp = sm + wrap5(sl + 1) * A.stage;
    float* N0 = sm + A.o_new + nl * rowsA * rp;
    const float* Nm = sm + A.o_new + wrap3(nl - 1) * rowsA * rp;
    // colour A of plane t on rows j0-1 .. j0+by
    if (doA) {
      const int par = (jj + t + A.c0) & 1;
      const float* rB0 = S0 + A.o_rB + offB;  // row jj of rho colour B, cell m0
      const float* pB0 = S0 + offB;
      float rc[4];
      unpack4(lds4(S0 + A.o_rA + offA), rc);
      float rxm[4], rxp[4], pxm[4], pxp[4];
      x_window(rB0 - 1 + par, pB0 - 1 + par, kZero, rxm, rxp, pxm, pxp);
      float rym[4], pym[4], ryp[4], pyp[4], rzm[4], pzm[4], rzp[4], pzp[4];
      nb_row(ym_ok ? rB0 - rp : wall_r + m0, ym_ok ? pB0 - rp : wall_p + m0, kZero, rym, pym);
      nb_row(yp_ok ? rB0 + rp : wall_r + m0, yp_ok ? pB0 + rp : wall_p + m0, kZero, ryp, pyp);
      const bool zm = t > 0, zp = t < A.nz - 1;
      nb_row(zm ? Sm + A.o_rB + offB : wall_r + m0, zm ? Sm + offB : wall_p + m0, kZero, rzm, pzm);
      nb_row(zp ? Sp + A.o_rB + offB : wall_r + m0, zp ? Sp + offB : wall_p + m0, kZero, rzp, pzp);
      const float4 v = relax4<kZero>(A, rc, bA, rxm, rxp, pxm, pxp, rym, pym, ryp, pyp, rzm, pzm,
                                     rzp, pzp);
      *reinterpret_cast<float4*>(N0 + offA) = v;
      if (own_row && t >= z0 && t < z1) *reinterpret_cast<float4*>(oA_p) = v;
    }
    __syncthreads();
    // colour B of plane u = t-1 on the block's rows, from the new colour A
    if (doB) {
      const float* Smm = sm + wrap5(sl - 2) * A.stage;
      const float* Nmm = sm + A.o_new + wrap3(nl - 2) * rowsA * rp;
      const int par = (jj + u + c1) & 1;
      float rc[4];
      unpack4(lds4(Sm + A.o_rB + offB), rc);
      const float* rA0 = Sm + A.o_rA + offA;  // row jj of rho colour A, plane u, cell m0
      const float* nA0 = Nm + offA;           // row jj of the new colour A, plane u
      float rxm[4], rxp[4], pxm[4], pxp[4];
      x_window(rA0 - 1 + par, nA0 - 1 + par, false, rxm, rxp, pxm, pxp);
      float rym[4], pym[4], ryp[4], pyp[4], rzm[4], pzm[4], rzp[4], pzp[4];
      nb_row(ym_ok ? rA0 - rp : wall_r + m0, ym_ok ? nA0 - rp : wall_p + m0, false, rym, pym);
      nb_row(yp_ok ? rA0 + rp : wall_r + m0, yp_ok ? nA0 + rp : wall_p + m0, false, ryp, pyp);
      const bool zm = u > 0, zp = u < A.nz - 1;
      nb_row(zm ? Smm + A.o_rA + offA : wall_r + m0, zm ? Nmm + offA : wall_p + m0, false, rzm,
             pzm);
      nb_row(zp ? S0 + A.o_rA + offA : wall_r + m0, zp ? N0 + offA : wall_p + m0, false, rzp, pzp);
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
  int by, threads, smem, rp, stage, o_rB, o_rA, o_new, o_wall;
};

// Rows per block for a row of hx half cells (hx <= 256): 16 rows up to 128
// half cells (576 threads at 128), 8 at 256 (640 threads).
SweepShape sweep_shape(int hx) {
  SweepShape S{};
  const int tq = hx / 4;
  S.by = hx <= 128 ? 16 : 8;
  S.threads = tq * (S.by + 2);
  S.rp = hx + 2 * kSwGuard;
  S.stage = S.rp * (2 * (S.by + 4) + (S.by + 2));
  S.stage = (S.stage + 31) & ~31;  // 128-byte aligned stages
  S.o_rB = S.rp * (S.by + 4);
  S.o_rA = 2 * S.rp * (S.by + 4);
  S.o_new = kSwStages * S.stage;
  S.o_wall = S.o_new + kSwNew * (S.by + 2) * S.rp;
  const size_t floats = (size_t)S.o_wall + 2 * (size_t)S.rp;
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
  return S.threads <= 640 && S.smem <= 227 * 1024;
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
  A.rp = S.rp; A.stage = S.stage; A.o_rB = S.o_rB; A.o_rA = S.o_rA; A.o_new = S.o_new;
  A.o_wall = S.o_wall;
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
