// The handle of the C ABI and the host helpers shared by its two translation
// units: gbmg.cu (the pressure solve, projection and adjoint) and ns_host.cu
// (the momentum step and the interface entry points).  Internal to the
// library; callers see only the opaque gbmg_handle of gbmg.h.
#pragma once

#include <cuda_runtime.h>

#include <string>

#include "gbmg.h"
#include "gbmg_internal.h"

namespace gbmg {


struct Level {
  int nx = 0, ny = 0, nz = 0;
  int fx = 1, fy = 1, fz = 1;
  size_t n = 0;
  double *cx = nullptr, *cy = nullptr, *cz = nullptr, *idiag = nullptr;
  double *sol = nullptr, *src = nullptr;  // owned on levels >= 1
  float *cx32 = nullptr, *cy32 = nullptr, *cz32 = nullptr;
  float *sol32 = nullptr, *src32 = nullptr;
  // FP32 kernels take the coefficients from this density instead of cx32..cz32
  // (finest level of a mixed solve whose operator came from rho or phi)
  const float* rho32 = nullptr;
  float k32[3] = {0.f, 0.f, 0.f};  // 2/h^2 per axis
  int split = 0;  // sol32, src32 and rho32 in the colour-split layout
  size_t hstride = 0;  // distance between the colour halves (elements)
  int zrev = 0;   // direction of the next split-kernel launch (toggles per launch)
};

enum GraphKind { kGraphNone = -1, kGraphFp64 = 0, kGraphMixed = 1, kGraphPcg64 = 2, kGraphPcgMixed = 3 };
constexpr int kGmresRestart = 30;   // flexible GMRES restart length
constexpr int kGmresBlocks = 1024;  // blocks of its dot-product kernel


}  // namespace gbmg

struct gbmg_handle {
  gbmg_grid grid{};
  gbmg_params prm{};
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  int L = 0;
  gbmg::Level lv[gbmg::kMaxLevels];
  size_t n0 = 0;
  bool mixed = false;
  // fine-level buffers
  double* b = nullptr;    // mean-free right-hand side
  double* p = nullptr;    // pressure being solved for
  double* rho = nullptr;  // cell density of the current operator
  float* rho32 = nullptr; // its FP32 copy (mixed precision)
  double* vel[3] = {nullptr, nullptr, nullptr};
  size_t vel_n[3] = {0, 0, 0};
  double* aux[2] = {nullptr, nullptr};  // adjoint outputs / staging, allocated on first use
  double* r0 = nullptr;  // initial FP64 residual of a warm-started mixed solve (first use)
  // flexible CG vectors (allocated when krylov = 1)
  double *kr = nullptr, *kz = nullptr, *kzold = nullptr, *kd = nullptr, *kq = nullptr;
  // flexible GMRES (krylov = 2): basis V (restart + 1 vectors), preconditioned
  // vectors Z (restart), dot partials, device and pinned host coefficients
  double *gmV = nullptr, *gmZ = nullptr, *gmPart = nullptr, *gmDev = nullptr, *gmHost = nullptr;
  // coarsest level
  int nc = 0;
  double *minv = nullptr, *adense = nullptr, *cwork = nullptr;
  float *minv32 = nullptr, *adense32 = nullptr;
  // reductions
  gbmg::ReduceScratch red{};
  double* host_res = nullptr;  // pinned mirror of red.result, then a copy of derr[0]
  int64_t flags_at = -1;       // launch count when derr[0] was last copied with the results
  int p_nonzero = -1;          // the initial p tested with the right-hand side (-1: not tested)
  // double-word finest level of the mixed solve: p (ping-pong), b, coefficients
  float2* pw[2] = {nullptr, nullptr};
  float2* bw = nullptr;
  float2 *cxw = nullptr, *cyw = nullptr, *czw = nullptr;
  int pcur = 0;  // which pw holds the current pressure
  int inner = 1;  // FP32 V-cycles per defect correction of the stationary mixed loop
  bool adaptive = false;  // ... the last correction as long as tail_cycles predicts
  cudaGraphExec_t tail_graph[4][2] = {};  // mixed iterations of 1 to 3 cycles (adaptive tail)
  int64_t tail_kernels[4][2] = {};
  // the split driver's stagnation test (set by gbmg_project_split): 0 off; 1 a
  // cycle that cuts the residual by under 1% (or raises it) ends the loop
  // (stagnated = true); 2 after the last restart: such a cycle ends it once
  // the residual is under 1000 tol
  int stag_mode = 0;
  bool stagnated = false;
  int sub_lc = 0;         // first level run by the one-block bottom of the cycle (L = none)
  int* derr = nullptr;   // device error flags (bulk-copy wait timeouts)
  gbmg::DefectMaps* dmaps = nullptr;  // TMA maps of the defect kernel: [p buffer][e: none,
                                      // the unknown], then [p buffer] with a colour-split e
  bool dmaps_split = false;     // whether the colour-split entries were made
  // captured iterations, per kind and per parity of pcur
  cudaGraphExec_t graph[4][2] = {};
  int64_t graph_kernels[4][2] = {};
  // the whole cycle loop as one graph (a device-side WHILE node), per kind and
  // per starting parity of pcur; loop_kernels: kernels per cycle
  cudaGraphExec_t loop_graph[4][2] = {};
  int64_t loop_kernels[4][2] = {};
  bool loop_off = false;          // the device loop could not be built: host loop
  gbmg::CycleCtl* ctl = nullptr;  // its state on the device, and a pinned mirror
  gbmg::CycleCtl* ctl_host = nullptr;
  // flexible GMRES: kz = M kr and kq = A kz as one captured graph
  cudaGraphExec_t gm_graph = nullptr;
  int64_t gm_graph_kernels = 0;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  // host transfers of a solve that overlap its kernels: the H2D of the initial
  // p beside the right-hand side's preparation, the D2H of the result beside
  // the FP64 certification
  cudaStream_t cstream = nullptr;
  // cev[0], cev[1]: ordering of the copy stream; cev[2]: the right-hand
  // side's upload; cev[3]: the staging buffer p free again (the operator
  // set-up from a host or device cell field leaves its later kernels running
  // after the call returns, once its input has been read); cev[4]: an input
  // field consumed
  cudaEvent_t cev[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
  const gbmg_field* dl_field = nullptr;  // set by gbmg_solve for solve_internal
  bool dl_started = false;
  int64_t launches = 0;
  // profiling: event pairs around launches, summed per kernel class
  bool prof = false;
  cudaEvent_t pev[2 * 512] = {};
  int pcls[512] = {};
  int pused = 0;
  double prof_ms[GBMG_PROF_CLASSES] = {};
  int64_t prof_n[GBMG_PROF_CLASSES] = {};
  bool coef_ready = false;
  bool fine_copies = false;  // finest FP32 / double-word coefficients already written
  bool rho_ready = false;
  bool split_ready = false;  // gbmg_set_split: constant Laplacian + density for the split source
  double split_rho12 = 0.0;
  // momentum step: padded-box buffers (vel%tmp, velsrc%tmp, and the host
  // staging copies of the caller's arrays), allocated on first use
  double* ns_buf[48] = {};
  size_t ns_n[48] = {};
  // CCD factor table of each axis is valid for these line lengths and spacings
  int ccd_L[3] = {0, 0, 0};
  double ccd_h[3] = {0.0, 0.0, 0.0};
  std::string err;
};

namespace gbmg {
namespace host {


#define GB_CUDA(h, call)                                                        \
  do {                                                                          \
    cudaError_t e_ = (call);                                                    \
    if (e_ != cudaSuccess) {                                                    \
      (h)->err = std::string(#call) + ": " + cudaGetErrorString(e_);            \
      return e_ == cudaErrorMemoryAllocation ? GBMG_OUT_OF_MEMORY : GBMG_CUDA_ERROR; \
    }                                                                           \
  } while (0)

#define GB_TRY(expr)            \
  do {                          \
    int rc_ = (expr);           \
    if (rc_ != GBMG_OK) return rc_; \
  } while (0)

inline int check_launch(gbmg_handle* h, const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    h->err = std::string(what) + ": " + cudaGetErrorString(e);
    return GBMG_CUDA_ERROR;
  }
  return GBMG_OK;
}

// Sum the recorded event pairs into the per-class totals (syncs the stream).
inline void prof_flush(gbmg_handle* h) {
  if (!h->pused) return;
  cudaStreamSynchronize(h->stream);
  for (int i = 0; i < h->pused; ++i) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, h->pev[2 * i], h->pev[2 * i + 1]) == cudaSuccess) {
      h->prof_ms[h->pcls[i]] += ms;
      h->prof_n[h->pcls[i]] += 1;
    }
  }
  h->pused = 0;
}

inline void prof_begin(gbmg_handle* h) {
  if (!h->prof) return;
  if (h->pused == 512) prof_flush(h);
  cudaEvent_t& e = h->pev[2 * h->pused];
  if (!e) cudaEventCreate(&e);
  cudaEventRecord(e, h->stream);
}

inline void prof_end(gbmg_handle* h, int cls) {
  h->launches += 1;
  if (!h->prof) return;
  cudaEvent_t& e = h->pev[2 * h->pused + 1];
  if (!e) cudaEventCreate(&e);
  cudaEventRecord(e, h->stream);
  h->pcls[h->pused++] = cls;
}

// One kernel launch, counted and (when profiling) timed as class `cls`.
#define LAUNCH(h, cls, stmt) \
  do {                       \
    prof_begin(h);           \
    stmt;                    \
    prof_end(h, cls);        \
  } while (0)

template <typename T>
inline int dmalloc(gbmg_handle* h, T** ptr, size_t n) {
  *ptr = nullptr;
  GB_CUDA(h, cudaMalloc((void**)ptr, (n ? n : 1) * sizeof(T)));
  return GBMG_OK;
}

template <typename T>
inline void dfree(T*& ptr) {
  if (ptr) cudaFree((void*)ptr);
  ptr = nullptr;
}

inline bool dense_cells(const gbmg_field& f, int nx, int ny) {
  return f.sy == nx && f.sz == (int64_t)nx * ny;
}

// Copy a field of extent (ex, ey, ez) into a dense device buffer.
inline int upload(gbmg_handle* h, const gbmg_field& f, int ex, int ey, int ez, int mem, double* dst,
           cudaStream_t s = nullptr) {
  if (!s) s = h->stream;
  if (!f.data) {
    h->err = "null field";
    return GBMG_INVALID_ARG;
  }
  const cudaMemcpyKind kind = mem == GBMG_MEM_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
  if (dense_cells(f, ex, ey)) {
    GB_CUDA(h, cudaMemcpyAsync(dst, f.data, (size_t)ex * ey * ez * sizeof(double), kind, s));
  } else if (mem == GBMG_MEM_DEVICE) {
    launch_copy_in(s, ex, ey, ez, Strided{f.data, f.sy, f.sz}, dst);
    h->launches += 1;
    GB_TRY(check_launch(h, "copy_in"));
  } else {
    for (int k = 0; k < ez; ++k)
      GB_CUDA(h, cudaMemcpy2DAsync(dst + (size_t)k * ex * ey, (size_t)ex * sizeof(double),
                                   f.data + (int64_t)k * f.sz, (size_t)f.sy * sizeof(double),
                                   (size_t)ex * sizeof(double), (size_t)ey, kind, s));
  }
  return GBMG_OK;
}

inline int download(gbmg_handle* h, const double* src, int ex, int ey, int ez, int mem,
             const gbmg_field& f, cudaStream_t s = nullptr) {
  if (!s) s = h->stream;
  const cudaMemcpyKind kind = mem == GBMG_MEM_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
  if (dense_cells(f, ex, ey)) {
    GB_CUDA(h, cudaMemcpyAsync(f.data, src, (size_t)ex * ey * ez * sizeof(double), kind, s));
  } else if (mem == GBMG_MEM_DEVICE) {
    launch_copy_out(s, ex, ey, ez, src, f.data, f.sy, f.sz);
    h->launches += 1;
    GB_TRY(check_launch(h, "copy_out"));
  } else {
    for (int k = 0; k < ez; ++k)
      GB_CUDA(h, cudaMemcpy2DAsync(f.data + (int64_t)k * f.sz, (size_t)f.sy * sizeof(double),
                                   src + (size_t)k * ex * ey, (size_t)ex * sizeof(double),
                                   (size_t)ex * sizeof(double), (size_t)ey, kind, s));
  }
  return GBMG_OK;
}


inline int validate_field(gbmg_handle* h, const gbmg_field& f, const char* name) {
  if (!f.data || f.sy < 1 || f.sz < 1) {
    h->err = std::string("invalid field ") + name;
    return GBMG_INVALID_ARG;
  }
  return GBMG_OK;
}

inline int begin(gbmg_handle* h) {
  if (!h) return GBMG_INVALID_ARG;
  h->err.clear();
  GB_CUDA(h, cudaSetDevice(h->device));
  return GBMG_OK;
}

// b = div(u*)/dt on the device face velocities, the solve from the initial
// pressure in h->p, and the correction (gbmg.cu)
int project_device(gbmg_handle* h, const gbmg_field dfield[3], bool has_w, double dt, double tol,
                   gbmg_stats* st);

}  // namespace host
}  // namespace gbmg
