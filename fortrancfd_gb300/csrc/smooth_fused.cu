// Fused red-black Gauss-Seidel sweep for the FP32 cycle (sm_103a).
//
// One launch does a whole sweep (red, then black) of one level, out of place:
// it reads p_in and writes p_out, so every block sees the same old values and
// the result equals the two-launch red/black sweep bit for bit, whatever the
// block schedule.  Each block owns a TX x TY tile of the x-y plane and marches
// up a chunk of z planes with a 4-plane ring of p in shared memory (tile plus
// a 2-cell halo).  At plane k it updates the red cells of plane k on the tile
// plus a 1-cell ring (the ring is recomputed by the neighbouring block too),
// then the black cells of plane k-1 on the tile, and stores plane k-1.  A sweep
// thus reads p, b and the three face-coefficient arrays once and writes p
// once: 24 bytes per cell in FP32 instead of about twice that for two
// colour launches.  Chunks of z start one plane early to recompute the red
// values under their first plane.
//
// Smoother of the reference's cycle: multigrid_relax
// ("DomainDecomposition/3D/src/others/multigrid_solver.f90:1-49"), with the
// variable-coefficient update p_i = (sum_f coe_f p_nb - b_i)/sum_f coe_f of
// ppe_sor_solver ("Two phase flows/newOpenMP/3D+IBM/src/ns_solver/
// ns_ppe_solver.f90:97-115").
#include <algorithm>

#include "gbmg_internal.h"

namespace gbmg {

namespace {

constexpr int kFTX = 64;     // tile width (x), two cells per thread
constexpr int kFTY = 8;      // tile height (y)
constexpr int kFZ = 32;      // default z planes per block
constexpr int kSX = kFTX + 4;
constexpr int kSY = kFTY + 4;
constexpr int kThreads = kFTX / 2 * kFTY;

template <typename T>
struct Ring {
  T p[4][kSY][kSX];
};

// Update one cell from the ring; returns the new value.  Neighbours outside
// the domain carry a zero coefficient and are not read.
template <typename T>
__device__ __forceinline__ T relax_cell(const LevelView<T>& L, const Ring<T>& R, int sk, int skm,
                                        int skp, int lx, int ly, int x, int y, int k) {
  const size_t sy = (size_t)L.nx, sz = (size_t)L.nx * L.ny;
  const size_t q = (size_t)k * sz + (size_t)y * sy + x;
  T s = T(0), d = T(0), c;
  if (x > 0) { c = __ldg(L.cx + q); s += c * R.p[sk][ly][lx - 1]; d += c; }
  if (x < L.nx - 1) { c = __ldg(L.cx + q + 1); s += c * R.p[sk][ly][lx + 1]; d += c; }
  if (y > 0) { c = __ldg(L.cy + q); s += c * R.p[sk][ly - 1][lx]; d += c; }
  if (y < L.ny - 1) { c = __ldg(L.cy + q + sy); s += c * R.p[sk][ly + 1][lx]; d += c; }
  if (k > 0) { c = __ldg(L.cz + q); s += c * R.p[skm][ly][lx]; d += c; }
  if (k < L.nz - 1) { c = __ldg(L.cz + q + sz); s += c * R.p[skp][ly][lx]; d += c; }
  return (s - __ldg(L.src + q)) / d;
}

template <typename T>
__device__ __forceinline__ void load_plane(const LevelView<T>& L, const T* __restrict__ pin,
                                           Ring<T>& R, int k, int x0, int y0, int tid) {
  const int slot = k & 3;
  const size_t sz = (size_t)L.nx * L.ny;
  for (int e = tid; e < kSX * kSY; e += kThreads) {
    const int lx = e % kSX, ly = e / kSX;
    const int x = x0 - 2 + lx, y = y0 - 2 + ly;
    T v = T(0);
    if (x >= 0 && x < L.nx && y >= 0 && y < L.ny) v = pin[(size_t)k * sz + (size_t)y * L.nx + x];
    R.p[slot][ly][lx] = v;
  }
}

// First-colour cells ((x+y+k)%2 == c0) of plane k on the tile plus a 1-cell
// ring, written into the ring.
template <typename T>
__device__ __forceinline__ void red_stage(const LevelView<T>& L, Ring<T>& R, int k, int x0, int y0,
                                          int tid, int c0) {
  constexpr int PX = kFTX / 2 + 1;  // cell pairs per extended row (x = -1 .. TX)
  constexpr int NY = kFTY + 2;
  const int sk = k & 3, skm = (k + 3) & 3, skp = (k + 1) & 3;
  for (int e = tid; e < PX * NY; e += kThreads) {
    const int px = e % PX, ey = e / PX;
    const int ly = 1 + ey, y = y0 - 1 + ey;
    // the pair covers lx = 1 + 2px and 2 + 2px; pick the first-colour one
    int lx = 1 + 2 * px;
    int x = x0 - 2 + lx;
    if (((x + y + k) & 1) != c0) { ++lx; ++x; }
    if (x < 0 || x >= L.nx || y < 0 || y >= L.ny || lx >= kSX - 1) continue;
    R.p[sk][ly][lx] = relax_cell(L, R, sk, skm, skp, lx, ly, x, y, k);
  }
}

template <typename T>
__global__ void __launch_bounds__(kThreads) k_smooth_fused(LevelView<T> L, const T* __restrict__ pin,
                                                           T* __restrict__ pout, int c0, int kz) {
  __shared__ Ring<T> R;
  const int tid = threadIdx.x;
  const int x0 = blockIdx.x * kFTX, y0 = blockIdx.y * kFTY;
  const int z0 = blockIdx.z * kz, z1 = min(z0 + kz, L.nz);
  // prologue: planes z0-2 .. z0, and red of plane z0-1 from them
  for (int k = max(z0 - 2, 0); k <= z0; ++k) load_plane(L, pin, R, k, x0, y0, tid);
  __syncthreads();
  if (z0 > 0) {
    red_stage(L, R, z0 - 1, x0, y0, tid, c0);
  }
  // the black-stage / store mapping: thread -> cell pair (2tx, 2tx+1) of row ty
  const int tx = tid % (kFTX / 2), ty = tid / (kFTX / 2);
  const int lx0 = 2 + 2 * tx, ly = 2 + ty;
  const int xa = x0 + 2 * tx, y = y0 + ty;
  for (int k = z0; k <= z1; ++k) {
    __syncthreads();
    // plane k+1 is read by the red stage of plane k, also at k = z1 (the
    // red values under the chunk's last black plane)
    if (k + 1 < L.nz) load_plane(L, pin, R, k + 1, x0, y0, tid);
    __syncthreads();
    if (k < L.nz && k <= z1) red_stage(L, R, k, x0, y0, tid, c0);
    __syncthreads();
    const int kb = k - 1;
    if (kb >= z0 && kb < z1 && y < L.ny) {
      const int sk = kb & 3, skm = (kb + 3) & 3, skp = (kb + 1) & 3;
      const size_t row = ((size_t)kb * L.ny + y) * L.nx;
#pragma unroll
      for (int c = 0; c < 2; ++c) {
        const int x = xa + c, lx = lx0 + c;
        if (x >= L.nx) continue;
        T v = R.p[sk][ly][lx];
        if (((x + y + kb) & 1) != c0) {
          v = relax_cell(L, R, sk, skm, skp, lx, ly, x, y, kb);
          R.p[sk][ly][lx] = v;
        }
        pout[row + x] = v;
      }
    }
  }
}

}  // namespace

template <typename T>
void launch_smooth_fused(cudaStream_t s, const LevelView<T>& L, const T* pin, T* pout,
                         int first_color, int planes) {
  const int kz = planes > 0 ? planes : kFZ;
  const dim3 grd((unsigned)((L.nx + kFTX - 1) / kFTX), (unsigned)((L.ny + kFTY - 1) / kFTY),
                 (unsigned)((L.nz + kz - 1) / kz));
  k_smooth_fused<T><<<grd, kThreads, 0, s>>>(L, pin, pout, first_color, kz);
}

template void launch_smooth_fused<float>(cudaStream_t, const LevelView<float>&, const float*,
                                         float*, int, int);

}  // namespace gbmg
