// Divergence statistics that allocate nothing: gbmg_div_stats_noalloc.
//
// gbmg_div_stats runs on a handle, and gbmg_create allocates the whole
// multigrid hierarchy (tens of bytes per cell) plus the reduction scratch on
// the device.  This entry point runs the same reduction kernel (k_div_stats,
// launched through launch_div_stats with the same block count, so the sums are
// taken in the same order) on the caller's device arrays, with its scratch in
// the file-scope __device__ array below: no handle, no cudaMalloc/cudaFree and
// no allocating library routine on any call.
//
// Scratch layout (doubles): kRedValues x kStaticBlocks per-block partial sums,
// then kRedSlots result slots, then one 8-byte slot holding the completion
// counter.  Only the counter must start at zero.  The block that finishes a
// reduction last resets it, but a launch that fails part-way can leave it
// non-zero, so every call zeroes it on the caller's stream before its launch
// (an 8-byte cudaMemsetAsync, which allocates nothing).  The partials are
// written before they are read, and launch_div_stats zeroes the max slot
// before every launch.
//
// Set-up: every call looks up the array's device address on the device it
// runs on (cudaGetSymbolAddress with that device current; a host-side lookup
// that allocates nothing).  The address is not cached: after a
// cudaDeviceReset the module is loaded again and the array may move.  The
// first call on a device may load the library's module there, so make it
// before any stream capture on that device.
//
// Overlapping calls race: every call on a device uses the one scratch, so two
// calls in flight at once (from two host threads, on any streams) corrupt each
// other's sums.  A call returns only after its stream has finished it, so
// calls from one host thread never overlap.
#include <climits>
#include <cstdio>

#include "gbmg.h"
#include "gbmg_internal.h"

namespace gbmg {
namespace {

// 8 blocks per SM (reduce_blocks_for) on devices of up to 256 SMs.
constexpr int kStaticBlocks = 2048;
constexpr size_t kStaticResult = (size_t)kRedValues * kStaticBlocks;
constexpr size_t kStaticCounter = kStaticResult + kRedSlots;
constexpr size_t kStaticDoubles = kStaticCounter + 1;  // 32,904 bytes

static __device__ __align__(256) double g_noalloc_scratch[kStaticDoubles];

void set_err(char* err, size_t len, const char* fmt, long long a = 0, long long b = 0) {
  if (err && len > 0) std::snprintf(err, len, fmt, a, b);
}

// Device address of the scratch on the current device, with its completion
// counter zeroed on stream s (ordered before the caller's launch on s).
int scratch_for(cudaStream_t s, double** out, char* err, size_t len) {
  void* p = nullptr;
  cudaError_t rc = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (rc != cudaSuccess || !p) {
    set_err(err, len, "div_stats_noalloc: cudaGetSymbolAddress failed (CUDA error %lld)", rc);
    return GBMG_CUDA_ERROR;
  }
  double* base = static_cast<double*>(p);
  rc = cudaMemsetAsync(base + kStaticCounter, 0, sizeof(double), s);
  if (rc != cudaSuccess) {
    set_err(err, len, "div_stats_noalloc: zeroing the completion counter failed (CUDA error %lld)",
            rc);
    return GBMG_CUDA_ERROR;
  }
  *out = base;
  return GBMG_OK;
}

bool field_ok(const gbmg_field& f) { return f.data && f.sy >= 1 && f.sz >= 1; }

}  // namespace
}  // namespace gbmg

using namespace gbmg;

extern "C" int gbmg_div_stats_noalloc(const gbmg_grid* grid, gbmg_field u, gbmg_field v,
                                      gbmg_field w, double* max_div, double* mean_div,
                                      int device, void* stream, char* err, size_t err_len) {
  if (err && err_len > 0) err[0] = '\0';
  if (!grid || grid->nx < 1 || grid->ny < 1 || grid->nz < 1 || !(grid->dx > 0) ||
      !(grid->dy > 0) || (grid->nz > 1 && !(grid->dz > 0))) {
    set_err(err, err_len, "div_stats_noalloc: invalid grid");
    return GBMG_INVALID_ARG;
  }
  if (!field_ok(u) || !field_ok(v)) {
    set_err(err, err_len, "div_stats_noalloc: invalid field u or v");
    return GBMG_INVALID_ARG;
  }
  // the kernel indexes rows (j, k) and x with 32-bit integers
  const long long rows = (long long)grid->ny * grid->nz;
  if (rows > INT_MAX || grid->nx >= INT_MAX) {
    set_err(err, err_len,
            "div_stats_noalloc: %lld rows of cells exceed the limit of %lld (2^31 - 1)", rows,
            (long long)INT_MAX);
    return GBMG_INVALID_ARG;
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
    cudaGetLastError();
    set_err(err, err_len, "div_stats_noalloc: no CUDA device");
    return GBMG_NO_DEVICE;
  }
  int prev = 0;
  cudaGetDevice(&prev);
  const int dev = device >= 0 ? device : prev;
  if (dev >= ndev) {
    set_err(err, err_len, "div_stats_noalloc: device %lld out of range (%lld devices)", dev,
            ndev);
    return GBMG_INVALID_ARG;
  }
  if (cudaSetDevice(dev) != cudaSuccess) {
    set_err(err, err_len, "div_stats_noalloc: cudaSetDevice(%lld) failed", dev);
    return GBMG_CUDA_ERROR;
  }
  const int blocks = reduce_blocks_for((size_t)rows);
  int st = GBMG_OK;
  if (blocks > kStaticBlocks) {
    set_err(err, err_len,
            "div_stats_noalloc: the reduction needs %lld blocks of partial sums, the static "
            "scratch holds %lld",
            blocks, kStaticBlocks);
    st = GBMG_INVALID_ARG;
  }
  const cudaStream_t s = static_cast<cudaStream_t>(stream);
  double* base = nullptr;
  if (st == GBMG_OK) st = scratch_for(s, &base, err, err_len);
  if (st == GBMG_OK) {
    const ReduceScratch R{base, reinterpret_cast<unsigned int*>(base + kStaticCounter),
                          base + kStaticResult, kStaticBlocks};
    const bool has_w = w.data != nullptr && grid->nz > 1;
    if (has_w && !field_ok(w)) {
      set_err(err, err_len, "div_stats_noalloc: invalid field w");
      st = GBMG_INVALID_ARG;
    } else {
      const Strided su{u.data, u.sy, u.sz}, sv{v.data, v.sy, v.sz};
      const Strided sw = has_w ? Strided{w.data, w.sy, w.sz} : Strided{nullptr, 0, 0};
      const double dz = grid->nz > 1 ? grid->dz : 1.0;
      launch_div_stats(s, grid->nx, grid->ny, grid->nz, su, sv, sw, grid->dx, grid->dy, dz, R);
      double res[kRedSlots];
      cudaError_t rc = cudaGetLastError();
      if (rc == cudaSuccess)
        rc = cudaMemcpyAsync(res, R.result, sizeof(res), cudaMemcpyDeviceToHost, s);
      if (rc == cudaSuccess) rc = cudaStreamSynchronize(s);
      if (rc != cudaSuccess) {
        set_err(err, err_len, "div_stats_noalloc: CUDA error %lld", rc);
        st = GBMG_CUDA_ERROR;
      } else {
        if (max_div) *max_div = res[kSlotMax];
        if (mean_div)
          *mean_div = res[kSlotSum] / (double)((size_t)grid->nx * grid->ny * grid->nz);
      }
    }
  }
  cudaSetDevice(prev);
  return st;
}
