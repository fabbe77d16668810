// Red-black Gauss-Seidel sweep fed by TMA, for the FP32 cycle (sm_103a).
//
// One launch = one whole sweep of one level, out of place (p_in -> p_out), so
// the result equals the two-colour-launch sweep bit for bit whatever the block
// schedule.  Blocks own a 64 x 8 tile of the x-y plane and march up a chunk of
// 32 z planes.  Thread 0 streams each plane's 72 x 12 boxes of p, b, cx, cy and
// cz (tile plus halo; the box starts at x0-4 so its x coordinate is 16-byte
// aligned) into a 5-slot shared-memory ring with cp.async.bulk.tensor, two
// planes ahead of the compute, completing on one mbarrier per slot.  At plane
// k the block updates the first colour of plane k on the tile plus a 1-cell
// ring (the ring is recomputed by the neighbour too), then the second colour
// of plane k-1 on the tile, and stores plane k-1.  TMA fills out-of-range box
// cells with zeros, and wall coefficients are stored as zeros, so the x and y
// walls need no branches.  HBM traffic per sweep: p, b, 3 coefficients read
// once, p written once (24 bytes per cell).
//
// Smoother of the reference's cycle, multigrid_relax
// ("DomainDecomposition/3D/src/others/multigrid_solver.f90:1-49"), with the
// variable-coefficient update of ppe_sor_solver ("Two phase flows/newOpenMP/
// 3D+IBM/src/ns_solver/ns_ppe_solver.f90:97-115").
#include <cudaTypedefs.h>

#include <algorithm>
#include <cstdlib>

#include "gbmg_internal.h"
#include "tma.cuh"

namespace gbmg {

namespace {

constexpr int kTX = 64, kTY = 8, kZC = 32;
constexpr int kBX = kTX + 8;  // box width, from x0 - 4
constexpr int kBY = kTY + 4;  // box height, from y0 - 2
constexpr int kTile = kBX * kBY;
constexpr int kSlots = 5;
constexpr int kArrays = 5;  // p, b, cx, cy, cz
constexpr int kThreads = kTX / 2 * kTY;
constexpr uint32_t kPlaneBytes = kArrays * kTile * sizeof(float);
constexpr size_t kSmemBytes = (size_t)kSlots * kPlaneBytes + 128 + kSlots * sizeof(uint64_t);

__device__ __forceinline__ float* tile(float* base, int slot, int a) {
  return base + ((size_t)slot * kArrays + a) * kTile;
}

// New value of the cell at box offset t of plane slot s (sm/sp: slots of the
// planes below/above; has_dn/has_up: whether those planes exist).  Order of
// the sums is x-, x+, y-, y+, z-, z+ as in the two-colour kernel.
__device__ __forceinline__ float relax(float* base, int s, int sm, int sp, bool has_dn, bool has_up,
                                      int t) {
  const float* P = tile(base, s, 0);
  const float* CX = tile(base, s, 2);
  const float* CY = tile(base, s, 3);
  float c, sum = 0.f, d = 0.f;
  c = CX[t];       sum += c * P[t - 1];   d += c;
  c = CX[t + 1];   sum += c * P[t + 1];   d += c;
  c = CY[t];       sum += c * P[t - kBX]; d += c;
  c = CY[t + kBX]; sum += c * P[t + kBX]; d += c;
  if (has_dn) { c = tile(base, s, 4)[t];  sum += c * tile(base, sm, 0)[t]; d += c; }
  if (has_up) { c = tile(base, sp, 4)[t]; sum += c * tile(base, sp, 0)[t]; d += c; }
  return (sum - tile(base, s, 1)[t]) / d;
}

__global__ void __launch_bounds__(kThreads, 2)
    k_smooth_tma(const __grid_constant__ SweepMaps maps, int nx, int ny, int nz, int zc,
                 float* __restrict__ pout, int c0, int* err) {
  extern __shared__ unsigned char smem_raw[];
  float* base = reinterpret_cast<float*>((reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~uintptr_t(127));
  uint64_t* bar = reinterpret_cast<uint64_t*>(base + (size_t)kSlots * kArrays * kTile);
  const int tid = threadIdx.x;
  const int x0 = blockIdx.x * kTX, y0 = blockIdx.y * kTY;
  const int z0 = blockIdx.z * zc, z1 = min(z0 + zc, nz);
  const int kstart = z0 > 0 ? z0 - 1 : z0;  // first plane whose first colour is computed
  const int kfirst_end = min(z1, nz - 1);   // last plane whose first colour is computed
  const int plo = max(kstart - 1, 0), phi = min(kfirst_end + 1, nz - 1);  // planes loaded
  if (tid == 0) {
    for (int s = 0; s < kSlots; ++s) mbar_init(&bar[s], 1);
    fence_barrier_init();
  }
  __syncthreads();

  auto issue = [&](int k) {  // thread 0
    const int s = k % kSlots;
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    mbar_arrive_expect_tx(&bar[s], kPlaneBytes);
    tma_load_3d(tile(base, s, 0), &maps.p, x0 - 4, y0 - 2, k, &bar[s]);
    tma_load_3d(tile(base, s, 1), &maps.b, x0 - 4, y0 - 2, k, &bar[s]);
    tma_load_3d(tile(base, s, 2), &maps.cx, x0 - 4, y0 - 2, k, &bar[s]);
    tma_load_3d(tile(base, s, 3), &maps.cy, x0 - 4, y0 - 2, k, &bar[s]);
    tma_load_3d(tile(base, s, 4), &maps.cz, x0 - 4, y0 - 2, k, &bar[s]);
  };

  uint32_t parity = 0;  // bit s = parity of the next phase of slot s
  const int pre_end = min(kstart + 1, phi);
  if (tid == 0)
    for (int k = plo; k <= pre_end; ++k) issue(k);
  int issued = pre_end, waited = plo - 1;

  const int tx = tid % (kTX / 2), ty = tid / (kTX / 2);
  for (int k = kstart; k <= z1; ++k) {
    if (k + 2 <= phi && k + 2 > issued) {
      if (tid == 0) issue(k + 2);
      issued = k + 2;
    }
    const int need = min(k + 1, phi);
    while (waited < need) {
      ++waited;
      const int s = waited % kSlots;
      mbar_wait(&bar[s], (parity >> s) & 1u, err);
      parity ^= 1u << s;
    }
    if (k <= kfirst_end) {
      // first colour of plane k on the tile plus a 1-cell ring
      const int s = k % kSlots, sm = (k + kSlots - 1) % kSlots, sp = (k + 1) % kSlots;
      const bool dn = k > 0, up = k < nz - 1;
      constexpr int PX = kTX / 2 + 1, NY = kTY + 2;
      for (int e = tid; e < PX * NY; e += kThreads) {
        const int px = e % PX, ey = e / PX;
        const int y = y0 - 1 + ey;
        int x = x0 - 1 + 2 * px;
        if (((x + y + k) & 1) != c0) ++x;
        if (x < 0 || x >= nx || y < 0 || y >= ny) continue;
        const int t = (ey + 1) * kBX + (x - x0 + 4);
        tile(base, s, 0)[t] = relax(base, s, sm, sp, dn, up, t);
      }
    }
    __syncthreads();
    const int kb = k - 1;
    if (kb >= z0 && kb < z1) {
      const int s = kb % kSlots, sm = (kb + kSlots - 1) % kSlots, sp = (kb + 1) % kSlots;
      const bool dn = kb > 0, up = kb < nz - 1;
      const int y = y0 + ty, xa = x0 + 2 * tx;
      if (y < ny && xa < nx) {
        float v[2];
#pragma unroll
        for (int c = 0; c < 2; ++c) {
          const int x = xa + c;
          const int t = (ty + 2) * kBX + (2 * tx + c + 4);
          v[c] = tile(base, s, 0)[t];
          if (x < nx && ((x + y + kb) & 1) != c0) v[c] = relax(base, s, sm, sp, dn, up, t);
        }
        float* row = pout + ((size_t)kb * ny + y) * nx;
        if (xa + 1 < nx && !(nx & 1)) {
          *reinterpret_cast<float2*>(row + xa) = make_float2(v[0], v[1]);
        } else {
          row[xa] = v[0];
          if (xa + 1 < nx) row[xa + 1] = v[1];
        }
      }
    }
    __syncthreads();
  }
}

}  // namespace

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

bool make_sweep_maps(SweepMaps* m, const float* p, const float* b, const float* cx,
                     const float* cy, const float* cz, int nx, int ny, int nz) {
  const CUtensorMapDataType f32 = CU_TENSOR_MAP_DATA_TYPE_FLOAT32;
  return make_tensor_map_3d(&m->p, p, f32, 4, nx, ny, nz, kBX, kBY) &&
         make_tensor_map_3d(&m->b, b, f32, 4, nx, ny, nz, kBX, kBY) &&
         make_tensor_map_3d(&m->cx, cx, f32, 4, nx, ny, nz, kBX, kBY) &&
         make_tensor_map_3d(&m->cy, cy, f32, 4, nx, ny, nz, kBX, kBY) &&
         make_tensor_map_3d(&m->cz, cz, f32, 4, nx, ny, nz, kBX, kBY);
}

int smooth_tma_init() {
  return cudaFuncSetAttribute(k_smooth_tma, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)kSmemBytes) == cudaSuccess
             ? 0
             : -1;
}

void launch_smooth_tma(cudaStream_t s, const SweepMaps& maps, int nx, int ny, int nz, float* pout,
                       int first_color, int* err) {
  static int zc = 0;
  if (zc == 0) {
    const char* e = std::getenv("GBMG_TMA_ZC");
    zc = e ? std::max(1, std::atoi(e)) : kZC;
  }
  const dim3 grd((unsigned)((nx + kTX - 1) / kTX), (unsigned)((ny + kTY - 1) / kTY),
                 (unsigned)((nz + zc - 1) / zc));
  k_smooth_tma<<<grd, kThreads, kSmemBytes, s>>>(maps, nx, ny, nz, zc, pout, first_color, err);
}

}  // namespace gbmg
