// Host orchestration and C ABI of the GB300 pressure-Poisson multigrid.
//
// One handle owns the device hierarchy of one grid: FP64 face coefficients on
// every level (plus 1/diagonal for the FP64 smoother), FP32 copies for the
// mixed-precision cycle, cycle vectors, the dense coarsest-level inverse and
// the reduction scratch.  A solve is a loop of cycles; each cycle (V-cycle,
// FP64 residual and its norm, and the 8-byte copy of the norm to pinned host
// memory) is captured once as a CUDA graph and replayed, and the host reads
// one scalar per cycle to decide whether to stop.
//
// Reference call shape: ppe_sor_init; ppe_sor_solver(tol) -> ns_momentum_correction
// ("Two phase flows/newOpenMP/3D+IBM/src/ns_solver/ns_ppe_solver.f90:1-205"),
// with the cycle of "DomainDecomposition/3D/src/others/multigrid_solver.f90"
// and the outer loop of ppe_mg_solver
// ("DomainDecomposition/3D/src/ns_solver/ns_ppe_mg_solver.f90:17-50").
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "gbmg.h"
#include "gbmg_internal.h"
#include "handle.h"

using namespace gbmg;
using namespace gbmg::host;


namespace {

// Level plan, the same rule as the oracle: every axis with more than one cell
// halves per level; auto mode stops at <= coarse_max cells or when an axis is
// odd; explicit levels require divisibility (manager_init,
// "DomainDecomposition/3D/lib/data/branches.f90:172-216").
int plan_levels(const gbmg_grid& g, int levels, int coarse_max, int dims[][3]) {
  int n[3] = {g.nx, g.ny, g.nz};
  int L = 1;
  dims[0][0] = n[0]; dims[0][1] = n[1]; dims[0][2] = n[2];
  for (;;) {
    if (levels > 0 && L >= levels) break;
    if (levels <= 0 && (long)n[0] * n[1] * n[2] <= coarse_max) break;
    bool ok = true, any = false;
    for (int a = 0; a < 3; ++a)
      if (n[a] > 1) { any = true; if (n[a] % 2) ok = false; }
    if (!ok || !any) {
      if (levels > 0) return -1;
      break;
    }
    for (int a = 0; a < 3; ++a)
      if (n[a] > 1) n[a] /= 2;
    if (L >= kMaxLevels) return -1;
    dims[L][0] = n[0]; dims[L][1] = n[1]; dims[L][2] = n[2];
    ++L;
  }
  return L;
}

LevelView<double> v64(const Level& l) {
  return LevelView<double>{l.nx, l.ny, l.nz, l.fx, l.fy, l.fz, l.cx, l.cy, l.cz, l.idiag, l.sol, l.src};
}
LevelView<float> v32(const Level& l) {
  LevelView<float> v{l.nx, l.ny, l.nz, l.fx, l.fy, l.fz, l.cx32, l.cy32, l.cz32, nullptr,
                     l.sol32, l.src32, l.rho32, l.k32[0], l.k32[1], l.k32[2], l.split,
                     l.hstride};
  return v;
}
template <typename T>
LevelView<T> view(const Level& l);
template <>
LevelView<double> view<double>(const Level& l) { return v64(l); }
template <>
LevelView<float> view<float>(const Level& l) { return v32(l); }

// The view for the next launch on level l: split levels alternate the z
// direction of their kernels launch by launch (an L2 hint; results do not
// depend on it).
template <typename T>
LevelView<T> view_next(Level& l);
template <>
LevelView<double> view_next<double>(Level& l) { return v64(l); }
template <>
LevelView<float> view_next<float>(Level& l) {
  LevelView<float> v = v32(l);
  if (l.split) {
    v.zrev = l.zrev;
    l.zrev ^= 1;
  }
  return v;
}

template <typename T> const T* minv_of(const gbmg_handle* h);
template <> const double* minv_of<double>(const gbmg_handle* h) { return h->minv; }
template <> const float* minv_of<float>(const gbmg_handle* h) { return h->minv32; }
template <typename T> const T* adense_of(const gbmg_handle* h);
template <> const double* adense_of<double>(const gbmg_handle* h) { return h->adense; }
template <> const float* adense_of<float>(const gbmg_handle* h) { return h->adense32; }

// One red-black sweep of level l: two colour launches in place.
// zero_guess: the level's values are taken as zero (its first sweep after the
// coarse unknown was started at zero, or the finest level of a correction
// cycle), so no memset is needed and the first colour does not read p.
template <typename T>
void sweep(gbmg_handle* h, int l, int first_color, bool zero_guess);

template <>
void sweep<double>(gbmg_handle* h, int l, int first_color, bool zero_guess) {
  const LevelView<double> V = v64(h->lv[l]);
  const int cs = l == 0 ? GBMG_PROF_SMOOTH_FINE : GBMG_PROF_SMOOTH_COARSE;
  LAUNCH(h, cs, launch_smooth<double>(h->stream, V, first_color, zero_guess));
  LAUNCH(h, cs, launch_smooth<double>(h->stream, V, 1 - first_color));
}

template <>
void sweep<float>(gbmg_handle* h, int l, int first_color, bool zero_guess) {
  Level& lv = h->lv[l];
  const int cs = l == 0 ? GBMG_PROF_SMOOTH_FINE : GBMG_PROF_SMOOTH_COARSE;
  LAUNCH(h, cs, launch_smooth<float>(h->stream, view_next<float>(lv), first_color, zero_guess));
  LAUNCH(h, cs, launch_smooth<float>(h->stream, view_next<float>(lv), 1 - first_color));
}

// Levels [h->sub_lc, L) as one single-block launch.
template <typename T>
SubCycle<T> make_subcycle(gbmg_handle* h, bool reverse) {
  SubCycle<T> S{};
  const int lc = h->sub_lc;
  S.nlev = h->L - lc;
  S.nu1 = h->prm.nu1;
  S.nu2 = h->prm.nu2;
  S.reverse = reverse ? 1 : 0;
  S.n_coarse = h->nc;
  int off = 0;
  for (int i = 0; i < S.nlev; ++i) {
    const LevelView<T> V = view<T>(h->lv[lc + i]);
    const auto log2_of = [](int v) {
      int l = 0;
      while ((1 << l) < v) ++l;
      return (1 << l) == v ? l : -1;
    };
    const int lx = log2_of(V.nx), ly = log2_of(V.ny);
    S.lv[i] = SubLevel<T>{V.nx, V.ny, V.nz, V.fx, V.fy, V.fz, V.cx, V.cy, V.cz,
                          (lx >= 0 && ly >= 0) ? lx : -1, (lx >= 0 && ly >= 0) ? ly : -1};
    S.off[i] = off;
    off += 5 * V.nx * V.ny * V.nz;  // sol, src and the three coefficient arrays
  }
  S.off[S.nlev] = off;
  const LevelView<T> V0 = view<T>(h->lv[lc]);
  S.src_in = V0.src;
  S.sol_out = V0.sol;
  S.minv = minv_of<T>(h);
  S.adense = adense_of<T>(h);
  return S;
}

// One V-cycle on the current level-0 (sol, src) of type T.  reverse_post runs
// the post-smoothing colours black-first (symmetric preconditioner for CG).
// zero_fine: the level-0 unknown starts at zero (correction and Krylov
// cycles); requires nu1 > 0, otherwise the caller zeroes it.
template <typename T>
int enqueue_vcycle(gbmg_handle* h, bool reverse_post, bool zero_fine) {
  const int L = h->L;
  const cudaStream_t s = h->stream;
  const bool pre = h->prm.nu1 > 0;
  const int top = std::min(h->sub_lc, L - 1);  // levels above the bottom block
  for (int l = 0; l < top; ++l) {
    for (int it = 0; it < h->prm.nu1; ++it)
      sweep<T>(h, l, 0, it == 0 && (l > 0 || zero_fine));
    LAUNCH(h, l == 0 ? GBMG_PROF_RESTRICT_FINE : GBMG_PROF_RESTRICT_COARSE,
           launch_restrict<T>(s, view_next<T>(h->lv[l]), view<T>(h->lv[l + 1]), !pre));
  }
  if (h->sub_lc < L) {
    LAUNCH(h, GBMG_PROF_COARSE_SOLVE, launch_subcycle<T>(s, make_subcycle<T>(h, reverse_post)));
  } else {
    const LevelView<T> C = view<T>(h->lv[L - 1]);
    LAUNCH(h, GBMG_PROF_COARSE_SOLVE,
           launch_coarse_solve<T>(s, h->nc, minv_of<T>(h), adense_of<T>(h), C.src, C.sol));
  }
  for (int l = top - 1; l >= 0; --l) {
    // A colour launch does not read its own colour's values (Gauss-Seidel
    // overwrites them), so the colour that the first post-smoothing launch
    // updates needs no correction: the split finest level corrects only the
    // other one.  Results are unchanged bit for bit.
    const int live = (l == 0 && h->prm.nu2 > 0) ? (reverse_post ? 0 : 1) : -1;
    LAUNCH(h, l == 0 ? GBMG_PROF_PROLONG_FINE : GBMG_PROF_PROLONG_COARSE,
           launch_prolong<T>(s, view_next<T>(h->lv[l]), view<T>(h->lv[l + 1]), live));
    for (int it = 0; it < h->prm.nu2; ++it) sweep<T>(h, l, reverse_post ? 1 : 0, false);
  }
  return check_launch(h, "v-cycle");
}

// Algorithmic HBM bytes of one V-cycle (each array touched once per kernel).
double vcycle_bytes(const gbmg_handle* h, int w) {
  double bytes = 0.0;
  const bool idiag = (w == 8);
  for (int l = 0; l < h->L - 1; ++l) {
    const double n = (double)h->lv[l].n, nc = (double)h->lv[l + 1].n;
    const double sweep = (idiag ? 7.0 : 6.0) * w * n;  // p r/w, b, cx, cy, cz (+ 1/diag)
    bytes += (h->prm.nu1 + h->prm.nu2) * sweep;
    bytes += 5.0 * w * n + 2.0 * w * nc;  // restrict: p, b, cx, cy, cz -> coarse b, sol
    bytes += 2.0 * w * n + w * nc;        // prolong: p r/w, coarse e
  }
  bytes += 2.0 * w * h->nc + (double)w * h->nc * h->nc;
  return bytes;
}

int reset_graphs(gbmg_handle* h) {
  for (int k = 0; k < 4; ++k)
    for (int par = 0; par < 2; ++par) {
      if (h->graph[k][par]) cudaGraphExecDestroy(h->graph[k][par]);
      h->graph[k][par] = nullptr;
      h->graph_kernels[k][par] = 0;
    }
  for (int k = 0; k < 4; ++k)
    for (int par = 0; par < 2; ++par) {
      if (h->tail_graph[k][par]) cudaGraphExecDestroy(h->tail_graph[k][par]);
      h->tail_graph[k][par] = nullptr;
      h->tail_kernels[k][par] = 0;
    }
  for (int k = 0; k < 4; ++k)
    for (int par = 0; par < 2; ++par) {
      if (h->loop_graph[k][par]) cudaGraphExecDestroy(h->loop_graph[k][par]);
      h->loop_graph[k][par] = nullptr;
      h->loop_kernels[k][par] = 0;
    }
  if (h->gm_graph) cudaGraphExecDestroy(h->gm_graph);
  h->gm_graph = nullptr;
  h->gm_graph_kernels = 0;
  return GBMG_OK;
}

DwOperator dw_op(const gbmg_handle* h) {
  const Level& f = h->lv[0];
  return DwOperator{f.nx, f.ny, f.nz, h->cxw, h->cyw, h->czw, h->bw};
}

// p_out = p_in + e, r32 = b - A p_out (double-word), |r|^2 -> slot; pc = p_in buffer.
void enqueue_defect(gbmg_handle* h, int pc, const float* e, float* r32, int slot) {
  const Level& f = h->lv[0];
  const bool split = f.split != 0;
  const size_t hs = split ? f.hstride : 0;
  if (h->dmaps && (!split || h->dmaps_split)) {
    const int mi = split && e ? 4 + pc : pc * 2 + (e ? 1 : 0);
    launch_defect_tma(h->stream, h->dmaps[mi], f.nx, f.ny, f.nz, e != nullptr, h->pw[1 - pc], r32,
                      h->red, slot, h->derr, hs);
  } else {
    launch_defect(h->stream, dw_op(h), h->pw[pc], h->pw[1 - pc], e, r32, h->red, slot, hs);
  }
}

int free_all(gbmg_handle* h) {
  reset_graphs(h);
  for (int l = 0; l < h->L; ++l) {
    Level& v = h->lv[l];
    dfree(v.cx); dfree(v.cy); dfree(v.cz); dfree(v.idiag);
    if (l > 0) { dfree(v.sol); dfree(v.src); }
    dfree(v.cx32); dfree(v.cy32); dfree(v.cz32); dfree(v.sol32); dfree(v.src32);
  }
  dfree(h->b); dfree(h->p); dfree(h->rho); dfree(h->rho32);
  dfree(h->pw[0]); dfree(h->pw[1]); dfree(h->bw); dfree(h->cxw); dfree(h->cyw); dfree(h->czw);
  for (int a = 0; a < 3; ++a) dfree(h->vel[a]);
  dfree(h->aux[0]); dfree(h->aux[1]); dfree(h->r0);
  dfree(h->kr); dfree(h->kz); dfree(h->kzold); dfree(h->kd); dfree(h->kq);
  dfree(h->gmV); dfree(h->gmZ); dfree(h->gmPart); dfree(h->gmDev);
  if (h->gmHost) cudaFreeHost(h->gmHost);
  dfree(h->minv); dfree(h->adense); dfree(h->cwork); dfree(h->minv32); dfree(h->adense32); dfree(h->derr);
  for (int i = 0; i < 48; ++i) dfree(h->ns_buf[i]);
  delete[] h->dmaps;
  h->dmaps = nullptr;
  dfree(h->red.partials); dfree(h->red.counter); dfree(h->red.result);
  if (h->host_res) cudaFreeHost(h->host_res);
  h->host_res = nullptr;
  dfree(h->ctl);
  if (h->ctl_host) cudaFreeHost(h->ctl_host);
  h->ctl_host = nullptr;
  for (int i = 0; i < 2 * 512; ++i)
    if (h->pev[i]) cudaEventDestroy(h->pev[i]);
  if (h->ev0) cudaEventDestroy(h->ev0);
  for (int i = 0; i < 5; ++i)
    if (h->cev[i]) cudaEventDestroy(h->cev[i]);
  if (h->cstream) cudaStreamDestroy(h->cstream);
  if (h->ev1) cudaEventDestroy(h->ev1);
  h->ev0 = h->ev1 = nullptr;
  if (h->own_stream && h->stream) cudaStreamDestroy(h->stream);
  h->stream = nullptr;
  return GBMG_OK;
}

// The one-block bottom of the cycle: the first level >= 1 with at most
// kSubMaxCells cells and at least one coarser level below it
// (GBMG_SUBCYCLE=0 runs those levels as separate launches instead).
template <typename T>
void setup_subcycle(gbmg_handle* h) {
  h->sub_lc = h->L;
  if (const char* e = std::getenv("GBMG_SUBCYCLE"))
    if (std::atoi(e) == 0) return;
  for (int l = 1; l + 1 < h->L; ++l)
    if (h->lv[l].n <= (size_t)kSubMaxCells && h->L - l <= kSubMaxLevels) {
      h->sub_lc = l;
      break;
    }
  if (h->sub_lc >= h->L) return;
  const SubCycle<T> S = make_subcycle<T>(h, false);
  const size_t smem = subcycle_smem<T>(S);
  if (smem > 200 * 1024 || subcycle_init<T>(smem) != 0) h->sub_lc = h->L;
}

// TMA maps of the double-word defect kernel (finest level with nx % 4 == 0;
// GBMG_TMA_DEFECT=0 keeps the plain-load defect kernel).
int setup_tma(gbmg_handle* h) {
  Level& f = h->lv[0];
  const char* ed = std::getenv("GBMG_TMA_DEFECT");
  if (f.nx % 4 == 0 && !(ed && std::atoi(ed) == 0) && defect_tma_init() == 0) {
    // [p buffer][e: none, the level's unknown]; then, per p buffer, the
    // colour-split e (entries 4, 5, made by set_rho_form)
    DefectMaps* m = new DefectMaps[6];
    bool ok = true;
    for (int pc = 0; pc < 2; ++pc)
      for (int ei = 0; ei < 2; ++ei)
        ok = ok && make_defect_maps(&m[pc * 2 + ei], h->pw[pc], ei ? f.sol32 : nullptr, h->bw,
                                    h->cxw, h->cyw, h->czw, f.nx, f.ny, f.nz, 0);
    if (ok) h->dmaps = m;
    else delete[] m;
  }
  return GBMG_OK;
}

int allocate(gbmg_handle* h) {
  int dims[kMaxLevels][3];
  const int L = plan_levels(h->grid, h->prm.levels, h->prm.coarse_max, dims);
  if (L < 1) {
    h->err = "grid cannot be coarsened to the requested level count";
    return GBMG_INVALID_ARG;
  }
  const int nc = dims[L - 1][0] * dims[L - 1][1] * dims[L - 1][2];
  if (nc > kMaxCoarse) {
    h->err = "coarsest level has " + std::to_string(nc) + " cells; the dense coarse solve takes at most " +
             std::to_string(kMaxCoarse) + " (use more levels or a grid with more factors of 2)";
    return GBMG_INVALID_ARG;
  }
  h->L = L;
  h->nc = nc;
  const bool need64 = !h->mixed || h->prm.krylov;
  for (int l = 0; l < L; ++l) {
    Level& v = h->lv[l];
    v.nx = dims[l][0]; v.ny = dims[l][1]; v.nz = dims[l][2];
    v.n = (size_t)v.nx * v.ny * v.nz;
    if (l + 1 < L) {
      v.fx = v.nx / dims[l + 1][0]; v.fy = v.ny / dims[l + 1][1]; v.fz = v.nz / dims[l + 1][2];
    } else {
      v.fx = v.fy = v.fz = 1;
    }
    GB_TRY(dmalloc(h, &v.cx, v.n));
    GB_TRY(dmalloc(h, &v.cy, v.n));
    GB_TRY(dmalloc(h, &v.cz, v.n));
    if (!h->mixed) GB_TRY(dmalloc(h, &v.idiag, v.n));
    if (l > 0 && !h->mixed) {
      GB_TRY(dmalloc(h, &v.sol, v.n));
      GB_TRY(dmalloc(h, &v.src, v.n));
    }
    if (h->mixed) {
      // the finest level's unknown and right-hand side may be stored
      // colour-split, with a pad between the halves
      const size_t nv = l == 0 ? v.n + kSplitPadMax : v.n;
      GB_TRY(dmalloc(h, &v.cx32, v.n));
      GB_TRY(dmalloc(h, &v.cy32, v.n));
      GB_TRY(dmalloc(h, &v.cz32, v.n));
      GB_TRY(dmalloc(h, &v.sol32, nv));
      GB_TRY(dmalloc(h, &v.src32, nv));
    }
  }
  (void)need64;
  h->n0 = h->lv[0].n;
  GB_TRY(dmalloc(h, &h->b, h->n0));
  GB_TRY(dmalloc(h, &h->p, h->n0));
  GB_TRY(dmalloc(h, &h->rho, h->n0));
  if (h->mixed) {
    GB_TRY(dmalloc(h, &h->rho32, h->n0 + kSplitPadMax));
    GB_TRY(dmalloc(h, &h->pw[0], h->n0));
    GB_TRY(dmalloc(h, &h->pw[1], h->n0));
    GB_TRY(dmalloc(h, &h->bw, h->n0));
    GB_TRY(dmalloc(h, &h->cxw, h->n0));
    GB_TRY(dmalloc(h, &h->cyw, h->n0));
    GB_TRY(dmalloc(h, &h->czw, h->n0));
  }
  // the FP64 increment rule keeps the previous cycle's p
  if (h->prm.stop_rule == GBMG_STOP_INCREMENT && !h->mixed) GB_TRY(dmalloc(h, &h->r0, h->n0));
  if (h->prm.krylov) {
    GB_TRY(dmalloc(h, &h->kr, h->n0));
    GB_TRY(dmalloc(h, &h->kz, h->n0));
    GB_TRY(dmalloc(h, &h->kzold, h->n0));
    GB_TRY(dmalloc(h, &h->kd, h->n0));
    GB_TRY(dmalloc(h, &h->kq, h->n0));
    if (h->prm.krylov == 2) {
      GB_TRY(dmalloc(h, &h->gmV, (size_t)(kGmresRestart + 1) * h->n0));
      GB_TRY(dmalloc(h, &h->gmZ, (size_t)kGmresRestart * h->n0));
      GB_TRY(dmalloc(h, &h->gmPart, (size_t)(kGmresRestart + 1) * kGmresBlocks));
      GB_TRY(dmalloc(h, &h->gmDev, (size_t)3 * (kGmresRestart + 1)));
      GB_CUDA(h, cudaMallocHost((void**)&h->gmHost, 3 * (kGmresRestart + 1) * sizeof(double)));
    }
  }
  GB_TRY(dmalloc(h, &h->minv, (size_t)nc * nc));
  GB_TRY(dmalloc(h, &h->adense, (size_t)nc * nc));
  GB_TRY(dmalloc(h, &h->cwork, (size_t)2 * nc * nc + nc));
  GB_TRY(dmalloc(h, &h->minv32, (size_t)nc * nc));
  GB_TRY(dmalloc(h, &h->adense32, (size_t)nc * nc));
  const size_t rows = (size_t)h->lv[0].ny * h->lv[0].nz;
  const dim3 dg = defect_grid(h->lv[0].nx, h->lv[0].ny, h->lv[0].nz);
  const int mb = std::max({reduce_blocks_for(rows), reduce_blocks_for(h->n0),
                           (int)(dg.x * dg.y * dg.z)});
  h->red.max_blocks = mb;
  GB_TRY(dmalloc(h, &h->red.partials, (size_t)kRedValues * mb));
  GB_TRY(dmalloc(h, &h->red.counter, 1));
  GB_TRY(dmalloc(h, &h->red.result, kRedSlots));
  GB_CUDA(h, cudaMemsetAsync(h->red.counter, 0, sizeof(unsigned int), h->stream));
  GB_CUDA(h, cudaMemsetAsync(h->red.result, 0, kRedSlots * sizeof(double), h->stream));
  GB_CUDA(h, cudaMallocHost((void**)&h->host_res, (kRedSlots + 1) * sizeof(double)));
  GB_TRY(dmalloc(h, &h->ctl, 1));
  GB_CUDA(h, cudaMallocHost((void**)&h->ctl_host, sizeof(CycleCtl)));
  GB_TRY(dmalloc(h, &h->derr, 4));
  GB_CUDA(h, cudaMemsetAsync(h->derr, 0, 4 * sizeof(int), h->stream));
  if (h->mixed) GB_TRY(setup_tma(h));
  if (h->mixed) setup_subcycle<float>(h);
  else setup_subcycle<double>(h);
  GB_CUDA(h, cudaEventCreate(&h->ev0));
  GB_CUDA(h, cudaStreamCreateWithFlags(&h->cstream, cudaStreamNonBlocking));
  for (int i = 0; i < 5; ++i) GB_CUDA(h, cudaEventCreateWithFlags(&h->cev[i], cudaEventDisableTiming));
  GB_CUDA(h, cudaEventRecord(h->cev[3], h->stream));
  GB_CUDA(h, cudaEventCreate(&h->ev1));
  GB_CUDA(h, cudaStreamSynchronize(h->stream));
  return GBMG_OK;
}


// Coarse levels, 1/diagonal, FP32 copies and the coarse inverse from the
// level-0 FP64 coefficients.
int build_hierarchy(gbmg_handle* h) {
  const cudaStream_t s = h->stream;
  // the coarse levels' FP32 copies come out of the coarsening
  for (int l = 1; l < h->L; ++l) {
    Level& c = h->lv[l];
    LAUNCH(h, GBMG_PROF_SETUP,
           launch_coarsen(s, v64(h->lv[l - 1]), c.cx, c.cy, c.cz, c.nx, c.ny, c.nz,
                          Float3Out{{c.cx32, c.cy32, c.cz32}}));
  }
  for (int l = 0; l < h->L; ++l) {
    Level& v = h->lv[l];
    if (v.idiag) LAUNCH(h, GBMG_PROF_SETUP, launch_idiag(s, v64(v), v.idiag));
    if (l == 0 && v.cx32 && !h->fine_copies) {
      LAUNCH(h, GBMG_PROF_SETUP, launch_to_float(s, v.cx, v.cx32, v.n));
      LAUNCH(h, GBMG_PROF_SETUP, launch_to_float(s, v.cy, v.cy32, v.n));
      LAUNCH(h, GBMG_PROF_SETUP, launch_to_float(s, v.cz, v.cz32, v.n));
    }
  }
  LAUNCH(h, GBMG_PROF_SETUP,
         launch_coarse_invert(s, v64(h->lv[h->L - 1]), h->minv, h->adense, h->minv32, h->adense32, h->cwork));
  if (h->mixed && !h->fine_copies) {
    const Level& f = h->lv[0];
    LAUNCH(h, GBMG_PROF_SETUP, launch_to_dw(s, f.cx, h->cxw, f.n));
    LAUNCH(h, GBMG_PROF_SETUP, launch_to_dw(s, f.cy, h->cyw, f.n));
    LAUNCH(h, GBMG_PROF_SETUP, launch_to_dw(s, f.cz, h->czw, f.n));
  }
  GB_TRY(check_launch(h, "hierarchy"));
  h->coef_ready = true;
  return GBMG_OK;
}

// Whether the FP32 finest-level kernels compute their coefficients from the
// density (an operator from rho/phi; GBMG_RHO_COEF=0 turns it off), and
// whether that level
// is stored colour-split (density form, nx even, x halved by the first
// coarsening, the level outside the single-block bottom; GBMG_SPLIT=0 turns
// it off).  Captured graphs hold the level views, so a change drops them.
void set_rho_form(gbmg_handle* h, bool on) {
  Level& f = h->lv[0];
  // (with the finest level inside the single-block bottom, sub_lc == 0, that
  // block reads stored coefficients and the density form has no user)
  bool want = on && h->mixed && h->sub_lc > 0;
  if (const char* e = std::getenv("GBMG_RHO_COEF"))
    if (std::atoi(e) == 0) want = false;
  bool split = want && f.nx % 2 == 0 && h->L > 1 && f.fx == 2 && h->sub_lc > 0;
  if (const char* e = std::getenv("GBMG_SPLIT"))
    if (std::atoi(e) == 0) split = false;
  // the halves sit n/2 + pad apart (pad a multiple of 4 floats: 16-byte
  // aligned halves for the bulk copies and TMA maps; not a power of two, so
  // same-offset accesses to both halves fall on different DRAM channels)
  const size_t pad = 4128;
  const size_t hs = split ? f.n / 2 + pad : 0;
  const float* r = want ? h->rho32 : nullptr;
  if (r != f.rho32 || (int)split != f.split || hs != f.hstride) reset_graphs(h);
  if (split && h->dmaps && hs != f.hstride) {
    // colour-split e maps (rows of nx/2 floats must be 16-byte multiples)
    bool oks = f.nx % 8 == 0;
    for (int pc = 0; pc < 2 && oks; ++pc)
      oks = make_defect_maps(&h->dmaps[4 + pc], h->pw[pc], f.sol32, h->bw, h->cxw, h->cyw, h->czw,
                             f.nx, f.ny, f.nz, hs);
    h->dmaps_split = oks;
  }
  f.rho32 = r;
  f.split = split ? 1 : 0;
  f.hstride = hs;
  const gbmg_grid& g = h->grid;
  f.k32[0] = (float)(2.0 / (g.dx * g.dx));
  f.k32[1] = (float)(2.0 / (g.dy * g.dy));
  f.k32[2] = (float)(2.0 / (g.dz * g.dz));
}

int set_rho_device(gbmg_handle* h, const double* bulk_rho) {
  const gbmg_grid& g = h->grid;
  Level& f = h->lv[0];
  h->split_ready = false;
  set_rho_form(h, true);
  // the FP32 finest-level coefficients are only read without the density form
  float* c32[3] = {f.cx32, f.cy32, f.cz32};
  float2* cw[3] = {h->cxw, h->cyw, h->czw};
  const bool want32 = h->mixed && !f.rho32;
  // (the mixed cycle's FP32 density comes out of the same pass)
  LAUNCH(h, GBMG_PROF_SETUP,
         launch_face_coef(h->stream, g.nx, g.ny, g.nz, g.dx * g.dx, g.dy * g.dy, g.dz * g.dz,
                          h->rho, f.cx, f.cy, f.cz, want32 ? c32 : nullptr,
                          h->mixed ? cw : nullptr, bulk_rho, h->mixed ? h->rho32 : nullptr,
                          f.split ? f.hstride : 0));
  h->fine_copies = h->mixed;
  GB_TRY(check_launch(h, "face_coef"));
  h->rho_ready = true;
  return build_hierarchy(h);
}

// The result slots and the device error flag to the host, one wait.
int read_results(gbmg_handle* h) {
  GB_CUDA(h, cudaMemcpyAsync(h->host_res, h->red.result, kRedSlots * sizeof(double),
                             cudaMemcpyDeviceToHost, h->stream));
  GB_CUDA(h, cudaMemcpyAsync(h->host_res + kRedSlots, h->derr, sizeof(int),
                             cudaMemcpyDeviceToHost, h->stream));
  GB_CUDA(h, cudaStreamSynchronize(h->stream));
  h->flags_at = h->launches;
  return GBMG_OK;
}

// b -> h->b with the mean removed (when asked); result[kSlotSumB+1] = |b|^2.
// h->b holds the right-hand side: project its mean out (when asked), make the
// double-word copy of the mixed solve, and return |b|.
// check_p: also test whether the initial p is zero (the stationary mixed
// loop's start), after p_ready, in the same wait as |b|.
int finish_rhs(gbmg_handle* h, double* bnorm, bool check_p = false,
               cudaEvent_t p_ready = nullptr) {
  const bool rm = h->prm.remove_rhs_mean != 0;
  if (rm) LAUNCH(h, GBMG_PROF_VECTOR, launch_sum_dw(h->stream, h->b, h->n0, h->red, kSlotSumB));
  // one pass: the shift, |b|^2, the double-word copy and (stationary mixed
  // loop) the first FP32 residual of a solve from p = 0
  const Level& f = h->lv[0];
  float* r32 = h->mixed && h->prm.krylov == 0 ? f.src32 : nullptr;
  LAUNCH(h, GBMG_PROF_VECTOR,
         launch_rhs_prep(h->stream, h->b, h->n0, h->red, rm ? kSlotSumB : -1, kSlotSumB + 1,
                         h->mixed ? h->bw : nullptr, r32, f.nx, f.ny, f.split ? f.hstride : 0));
  GB_TRY(check_launch(h, "rhs"));
  const bool test_p = check_p && h->mixed && h->prm.krylov == 0;
  if (test_p) {
    if (p_ready) GB_CUDA(h, cudaStreamWaitEvent(h->stream, p_ready, 0));
    LAUNCH(h, GBMG_PROF_VECTOR, launch_nonzero(h->stream, h->p, h->n0, h->red.result + kSlotSum + 1));
    GB_TRY(check_launch(h, "initial guess"));
  }
  GB_TRY(read_results(h));
  *bnorm = std::sqrt(h->host_res[kSlotSumB + 1]);
  h->p_nonzero = -1;
  if (test_p) {
    unsigned long long nz = 0ull;
    std::memcpy(&nz, &h->host_res[kSlotSum + 1], sizeof(nz));
    h->p_nonzero = nz != 0ull ? 1 : 0;
  }
  return GBMG_OK;
}

int read_result(gbmg_handle* h, int slot, double* v) {
  GB_TRY(read_results(h));
  *v = h->host_res[slot];
  return GBMG_OK;
}

// Enqueue the body of one solver iteration for the given kind.
// cycles: FP32 V-cycles of a mixed iteration (one defect correction)
int enqueue_iteration(gbmg_handle* h, int kind, bool first, bool to_host = true, int cycles = 1) {
  const cudaStream_t s = h->stream;
  Level& f = h->lv[0];
  const size_t n = h->n0;
  const int V = GBMG_PROF_VECTOR, R = GBMG_PROF_RESIDUAL;
  const bool zg = h->prm.nu1 > 0;  // zero initial guess handled by the first sweep
  const bool inc = h->prm.stop_rule == GBMG_STOP_INCREMENT;
  if (kind == kGraphFp64) {
    f.sol = h->p; f.src = h->b;
    // the increment rule compares p after the cycle with p before it
    if (inc) GB_CUDA(h, cudaMemcpyAsync(h->r0, h->p, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
    GB_TRY(enqueue_vcycle<double>(h, false, false));
    if (inc) LAUNCH(h, V, launch_increment<double>(s, h->p, h->r0, n, 0, h->red, kSlotIncSum, kSlotInc));
    LAUNCH(h, R, launch_residual_norm<double>(s, v64(f), (double*)nullptr, h->red, kSlotNorm));
  } else if (kind == kGraphMixed) {
    // e = V-cycles(r) in FP32 (the first from zero, the others continuing
    // from e); p += e and r = b - A p in double-word
    if (!zg) GB_CUDA(h, cudaMemsetAsync(f.sol32, 0, n * sizeof(float), s));
    GB_TRY(enqueue_vcycle<float>(h, false, zg));
    for (int c = 1; c < cycles; ++c) GB_TRY(enqueue_vcycle<float>(h, false, false));
    // the increment rule: the cycle's correction e is p_k - p_(k-1)
    if (inc)
      LAUNCH(h, V, launch_increment<float>(s, f.sol32, (const float*)nullptr, n,
                                           f.split ? f.hstride : 0, h->red, kSlotIncSum, kSlotInc));
    LAUNCH(h, R, enqueue_defect(h, h->pcur, f.sol32, f.src32, kSlotNorm));
  } else {
    // flexible CG: z = M r (one V-cycle from zero), mean-free
    if (kind == kGraphPcg64) {
      if (!zg) GB_CUDA(h, cudaMemsetAsync(h->kz, 0, n * sizeof(double), s));
      f.sol = h->kz; f.src = h->kr;
      GB_TRY(enqueue_vcycle<double>(h, true, zg));
    } else {
      if (f.split) LAUNCH(h, V, launch_to_split(s, h->kr, f.src32, f.nx, f.ny, f.nz, f.hstride));
      else LAUNCH(h, V, launch_double_to_float(s, h->kr, f.src32, n));
      if (!zg) GB_CUDA(h, cudaMemsetAsync(f.sol32, 0, n * sizeof(float), s));
      GB_TRY(enqueue_vcycle<float>(h, true, zg));
      if (f.split)
        LAUNCH(h, V, launch_from_split(s, f.sol32, h->kz, f.nx, f.ny, f.nz, f.hstride));
      else LAUNCH(h, V, launch_float_to_double(s, f.sol32, h->kz, n));
    }
    LAUNCH(h, V, launch_sum(s, h->kz, n, h->red, kSlotSum));
    LAUNCH(h, V, launch_shift_by_mean(s, h->kz, h->kz, n, h->red, kSlotSum, -1));
    LAUNCH(h, V, launch_dot2(s, h->kr, h->kz, h->kzold, n, h->red, kSlotDot));
    LAUNCH(h, V, launch_pcg_direction(s, h->kd, h->kzold, h->kz, n, h->red, first ? 1 : 0));
    h->launches += 1;  // the one-thread rz bookkeeping kernel
    f.sol = h->p; f.src = h->b;
    LAUNCH(h, R, launch_apply_dot(s, v64(f), h->kd, h->kq, h->red, kSlotDot2));
    LAUNCH(h, V, launch_pcg_step(s, h->p, h->kd, n, h->red));
    LAUNCH(h, R, launch_residual_norm<double>(s, v64(f), h->kr, h->red, kSlotNorm));
  }
  if (to_host)
    GB_CUDA(h, cudaMemcpyAsync(h->host_res, h->red.result, kRedSlots * sizeof(double),
                               cudaMemcpyDeviceToHost, s));
  return check_launch(h, "iteration");
}

int run_iteration(gbmg_handle* h, int kind, bool first, int cycles = 1) {
  // (mixed iterations of another length than inner: graphs for 1 to 3
  // cycles, the adaptive tail; eager otherwise)
  const bool tail = kind == kGraphMixed && cycles != h->inner;
  if (!h->prm.use_graph || first || h->prof || (tail && cycles > 3)) {
    GB_TRY(enqueue_iteration(h, kind, first, true, cycles));
    return GBMG_OK;
  }
  const int par = kind == kGraphMixed ? h->pcur : 0;
  cudaGraphExec_t& gx = tail ? h->tail_graph[cycles][par] : h->graph[kind][par];
  int64_t& gk = tail ? h->tail_kernels[cycles][par] : h->graph_kernels[kind][par];
  if (!gx) {
    cudaGraph_t g = nullptr;
    const int64_t before = h->launches;
    GB_CUDA(h, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    const int rc = enqueue_iteration(h, kind, false, true, cycles);
    const cudaError_t ec = cudaStreamEndCapture(h->stream, &g);
    if (rc != GBMG_OK) {
      if (g) cudaGraphDestroy(g);
      return rc;
    }
    if (ec != cudaSuccess) {
      h->err = std::string("graph capture: ") + cudaGetErrorString(ec);
      if (g) cudaGraphDestroy(g);
      return GBMG_CUDA_ERROR;
    }
    gk = h->launches - before;
    h->launches = before;
    const cudaError_t ei = cudaGraphInstantiate(&gx, g, 0);
    cudaGraphDestroy(g);
    if (ei != cudaSuccess) {
      h->err = std::string("graph instantiate: ") + cudaGetErrorString(ei);
      gx = nullptr;
      return GBMG_CUDA_ERROR;
    }
  }
  GB_CUDA(h, cudaGraphLaunch(gx, h->stream));
  h->launches += gk;
  return GBMG_OK;
}

// The cycle loop as one graph: a WHILE node whose body is the iteration of
// `kind` followed by k_cycle_ctl, which applies the stopping tests on the
// device and ends the loop, so the host waits once per solve instead of once
// per cycle.  The mixed iteration alternates its two p buffers, so its body is
// the iteration from buffer par, the controller, then (an IF node on that
// controller's decision) the iteration from the other buffer and the
// controller again.  Leaves h->loop_graph[kind][par] null, and sets
// h->loop_off, when the graph cannot be built (the host loop then runs).
int build_loop(gbmg_handle* h, int kind, int par) {
  const cudaStream_t s = h->stream;
  const bool two = kind == kGraphMixed;
  const int step = two ? h->inner : 1;
  cudaGraph_t g = nullptr;
  GB_CUDA(h, cudaGraphCreate(&g, 0));
  const int64_t before = h->launches;
  const int pcur = h->pcur;
  int rc = GBMG_OK;
  bool capturing = false;
  cudaError_t e = cudaSuccess;
  cudaGraph_t done = nullptr;
  do {
    cudaGraphConditionalHandle hw{}, hi{};
    if ((e = cudaGraphConditionalHandleCreate(&hw, g, 1, cudaGraphCondAssignDefault))) break;
    cudaGraphNodeParams wp{};
    wp.type = cudaGraphNodeTypeConditional;
    wp.conditional.handle = hw;
    wp.conditional.type = cudaGraphCondTypeWhile;
    wp.conditional.size = 1;
    cudaGraphNode_t wn = nullptr;
    if ((e = cudaGraphAddNode(&wn, g, nullptr, nullptr, 0, &wp))) break;
    cudaGraph_t body = wp.conditional.phGraph_out[0];
    if (two && (e = cudaGraphConditionalHandleCreate(&hi, body, 0, 0))) break;
    if ((e = cudaStreamBeginCaptureToGraph(s, body, nullptr, nullptr, 0,
                                           cudaStreamCaptureModeThreadLocal)))
      break;
    capturing = true;
    h->pcur = par;
    if ((rc = enqueue_iteration(h, kind, false, false, step)) != GBMG_OK) break;
    launch_cycle_ctl(s, h->ctl, h->red.result, hw, hi, two ? 1 : 0);
    h->launches += 1;
    if (two) {
      cudaStreamCaptureStatus cs;
      const cudaGraphNode_t* d = nullptr;
      size_t nd = 0;
      if ((e = cudaStreamGetCaptureInfo(s, &cs, nullptr, nullptr, &d, nullptr, &nd))) break;
      std::vector<cudaGraphNode_t> deps(d, d + nd);
      capturing = false;
      if ((e = cudaStreamEndCapture(s, &done))) break;
      cudaGraphNodeParams ip{};
      ip.type = cudaGraphNodeTypeConditional;
      ip.conditional.handle = hi;
      ip.conditional.type = cudaGraphCondTypeIf;
      ip.conditional.size = 1;
      cudaGraphNode_t in = nullptr;
      if ((e = cudaGraphAddNode(&in, body, deps.data(), nullptr, deps.size(), &ip))) break;
      if ((e = cudaStreamBeginCaptureToGraph(s, ip.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                             cudaStreamCaptureModeThreadLocal)))
        break;
      capturing = true;
      h->pcur = 1 - par;
      if ((rc = enqueue_iteration(h, kind, false, false, step)) != GBMG_OK) break;
      launch_cycle_ctl(s, h->ctl, h->red.result, hw, hi, 0);
      h->launches += 1;
    }
    capturing = false;
    if ((e = cudaStreamEndCapture(s, &done))) break;
    if ((e = cudaGraphInstantiate(&h->loop_graph[kind][par], g, 0))) {
      h->loop_graph[kind][par] = nullptr;
      break;
    }
  } while (false);
  if (capturing) cudaStreamEndCapture(s, &done);
  h->pcur = pcur;
  h->loop_kernels[kind][par] = (h->launches - before) / (two ? 2 : 1);
  h->launches = before;
  cudaGraphDestroy(g);
  if (rc != GBMG_OK) return rc;
  if (e != cudaSuccess || !h->loop_graph[kind][par]) {
    cudaGetLastError();
    h->loop_off = true;
  }
  return GBMG_OK;
}

// Runs cycles on the device from the state *c until the stopping tests end
// them; *c receives the final state.  *used = false: the device loop is not
// available and nothing ran.
int run_loop(gbmg_handle* h, int kind, CycleCtl* c, bool* used) {
  *used = false;
  if (h->loop_off || h->prm.use_graph != 1 || h->prof || h->stag_mode) return GBMG_OK;
  const int par = kind == kGraphMixed ? h->pcur : 0;
  if (!h->loop_graph[kind][par]) {
    GB_TRY(build_loop(h, kind, par));
    if (!h->loop_graph[kind][par]) return GBMG_OK;
  }
  const cudaStream_t s = h->stream;
  const int it0 = c->iters;
  *h->ctl_host = *c;
  GB_CUDA(h, cudaMemcpyAsync(h->ctl, h->ctl_host, sizeof(CycleCtl), cudaMemcpyHostToDevice, s));
  GB_CUDA(h, cudaGraphLaunch(h->loop_graph[kind][par], s));
  GB_CUDA(h, cudaMemcpyAsync(h->ctl_host, h->ctl, sizeof(CycleCtl), cudaMemcpyDeviceToHost, s));
  GB_CUDA(h, cudaMemcpyAsync(h->host_res, h->red.result, kRedSlots * sizeof(double),
                             cudaMemcpyDeviceToHost, s));
  GB_CUDA(h, cudaMemcpyAsync(h->host_res + kRedSlots, h->derr, sizeof(int),
                             cudaMemcpyDeviceToHost, s));
  GB_CUDA(h, cudaStreamSynchronize(s));
  *c = *h->ctl_host;
  h->launches += h->loop_kernels[kind][par] * (int64_t)(c->iters - it0);
  h->flags_at = h->launches;
  *used = true;
  return GBMG_OK;
}

// The solve loop on the internal (b, p).  Leaves p mean-free.
// z = M v: one V-cycle from zero on v (the flexible-CG preconditioner),
// mean-free.  Leaves the finest level's sol/src pointing at p and b.
int precondition(gbmg_handle* h, const double* v, double* z) {
  const cudaStream_t s = h->stream;
  Level& f = h->lv[0];
  const size_t n = h->n0;
  const int V = GBMG_PROF_VECTOR;
  const bool zg = h->prm.nu1 > 0;
  if (!h->mixed) {
    if (!zg) GB_CUDA(h, cudaMemsetAsync(z, 0, n * sizeof(double), s));
    f.sol = z; f.src = const_cast<double*>(v);
    GB_TRY(enqueue_vcycle<double>(h, true, zg));
  } else {
    if (f.split) LAUNCH(h, V, launch_to_split(s, v, f.src32, f.nx, f.ny, f.nz, f.hstride));
    else LAUNCH(h, V, launch_double_to_float(s, v, f.src32, n));
    if (!zg) GB_CUDA(h, cudaMemsetAsync(f.sol32, 0, n * sizeof(float), s));
    GB_TRY(enqueue_vcycle<float>(h, true, zg));
    if (f.split) LAUNCH(h, V, launch_from_split(s, f.sol32, z, f.nx, f.ny, f.nz, f.hstride));
    else LAUNCH(h, V, launch_float_to_double(s, f.sol32, z, n));
  }
  LAUNCH(h, V, launch_sum(s, z, n, h->red, kSlotSum));
  LAUNCH(h, V, launch_shift_by_mean(s, z, z, n, h->red, kSlotSum, -1));
  f.sol = h->p; f.src = h->b;
  return check_launch(h, "preconditioner");
}

// kz = M kr, kq = A kz: enqueued, or replayed from a graph captured on first use
int gm_apply(gbmg_handle* h) {
  const cudaStream_t s = h->stream;
  Level& f = h->lv[0];
  const auto enqueue = [&]() -> int {
    GB_TRY(precondition(h, h->kr, h->kz));
    LAUNCH(h, GBMG_PROF_RESIDUAL, launch_apply_dot(s, v64(f), h->kz, h->kq, h->red, kSlotDot2));
    return check_launch(h, "preconditioned product");
  };
  if (!h->prm.use_graph || h->prof) return enqueue();
  if (!h->gm_graph) {
    cudaGraph_t g = nullptr;
    const int64_t before = h->launches;
    GB_CUDA(h, cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    const int rc = enqueue();
    const cudaError_t ec = cudaStreamEndCapture(s, &g);
    if (rc != GBMG_OK || ec != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      if (rc != GBMG_OK) return rc;
      h->err = std::string("graph capture: ") + cudaGetErrorString(ec);
      return GBMG_CUDA_ERROR;
    }
    h->gm_graph_kernels = h->launches - before;
    h->launches = before;
    const cudaError_t ei = cudaGraphInstantiate(&h->gm_graph, g, 0);
    cudaGraphDestroy(g);
    if (ei != cudaSuccess) {
      h->gm_graph = nullptr;
      h->err = std::string("graph instantiate: ") + cudaGetErrorString(ei);
      return GBMG_CUDA_ERROR;
    }
  }
  GB_CUDA(h, cudaGraphLaunch(h->gm_graph, s));
  h->launches += h->gm_graph_kernels;
  return GBMG_OK;
}

// Flexible GMRES(kGmresRestart) around the V-cycle (right preconditioning,
// Saad's FGMRES): the residual norm falls monotonically, where conjugate
// gradients can first raise it many-fold on a smooth right-hand side (the
// adjoint of a smooth objective).  Per Arnoldi step: z_j = M v_j and
// w = A z_j (one captured graph on fixed buffers: v_j is copied in, z_j out),
// classical Gram-Schmidt on the device with a second pass only when the
// first removed most of w, one copy of the coefficients to the host for the
// Givens rotations, and w scaled into v_{j+1}.  At each restart and at the end the true FP64 residual b - A p
// is recomputed.  On entry kr holds r0 = b - A p and host_res[kSlotNorm] its
// squared norm.
int fgmres(gbmg_handle* h, double tol, double scale, double* rel_io, int* cycles, int* status) {
  const cudaStream_t s = h->stream;
  Level& f = h->lv[0];
  const size_t n = h->n0;
  const int m = kGmresRestart;
  const int VC = GBMG_PROF_VECTOR;
  const size_t bytes = n * sizeof(double);
  double* h1 = h->gmDev;               // first Gram-Schmidt pass
  double* h2 = h->gmDev + (m + 1);     // second pass
  double* nrm = h->gmDev + 2 * (m + 1);  // |w|^2 after, then before, the first pass
  std::vector<double> H((size_t)(m + 1) * m, 0.0), cs(m), sn(m), g(m + 1), y(m), col(m + 1);
  double r2 = h->host_res[kSlotNorm];
  double rel = *rel_io;
  int total = 0;
  *status = GBMG_NOT_CONVERGED;
  while (total < h->prm.max_cycles) {
    const double beta = std::sqrt(r2);
    if (!(beta > 0.0)) { *status = GBMG_OK; break; }
    LAUNCH(h, VC, launch_scale_copy(s, h->gmV, h->kr, 1.0 / beta, n));
    std::fill(g.begin(), g.end(), 0.0);
    g[0] = beta;
    int j = 0;
    for (; j < m && total < h->prm.max_cycles;) {
      double* vj = h->gmV + (size_t)j * n;
      double* w = h->kq;  // A z_j, orthogonalised in place, then scaled into V_{j+1}
      GB_CUDA(h, cudaMemcpyAsync(h->kr, vj, bytes, cudaMemcpyDeviceToDevice, s));
      GB_TRY(gm_apply(h));
      GB_CUDA(h, cudaMemcpyAsync(h->gmZ + (size_t)j * n, h->kz, bytes, cudaMemcpyDeviceToDevice, s));
      // classical Gram-Schmidt; a second pass only when the first removed most
      // of w (|w| fell below 0.7 of its length: "twice is enough")
      LAUNCH(h, VC, launch_mdot(s, w, n, 1, w, n, h->gmPart, kGmresBlocks, nrm + 1));
      LAUNCH(h, VC, launch_mdot(s, h->gmV, n, j + 1, w, n, h->gmPart, kGmresBlocks, h1));
      LAUNCH(h, VC, launch_maxpy(s, w, h->gmV, n, h1, j + 1, -1.0, n));
      LAUNCH(h, VC, launch_mdot(s, w, n, 1, w, n, h->gmPart, kGmresBlocks, nrm));
      h->launches += 3;  // the finishing kernels of the dot launches
      GB_CUDA(h, cudaMemcpyAsync(h->gmHost, h->gmDev, 3 * (m + 1) * sizeof(double),
                                 cudaMemcpyDeviceToHost, s));
      GB_CUDA(h, cudaStreamSynchronize(s));
      GB_TRY(check_launch(h, "arnoldi"));
      for (int i = 0; i <= j; ++i) col[i] = h->gmHost[i];
      double hn = std::sqrt(h->gmHost[2 * (m + 1)]);
      const double before = std::sqrt(h->gmHost[2 * (m + 1) + 1]);
      if (hn < 0.7 * before) {
        LAUNCH(h, VC, launch_mdot(s, h->gmV, n, j + 1, w, n, h->gmPart, kGmresBlocks, h2));
        LAUNCH(h, VC, launch_maxpy(s, w, h->gmV, n, h2, j + 1, -1.0, n));
        LAUNCH(h, VC, launch_mdot(s, w, n, 1, w, n, h->gmPart, kGmresBlocks, nrm));
        h->launches += 2;
        GB_CUDA(h, cudaMemcpyAsync(h->gmHost, h->gmDev, 3 * (m + 1) * sizeof(double),
                                   cudaMemcpyDeviceToHost, s));
        GB_CUDA(h, cudaStreamSynchronize(s));
        GB_TRY(check_launch(h, "arnoldi"));
        for (int i = 0; i <= j; ++i) col[i] += h->gmHost[(m + 1) + i];
        hn = std::sqrt(h->gmHost[2 * (m + 1)]);
      }
      col[j + 1] = hn;
      LAUNCH(h, VC, launch_scale_copy(s, h->gmV + (size_t)(j + 1) * n, w, hn > 0.0 ? 1.0 / hn : 0.0,
                                      n));
      for (int i = 0; i < j; ++i) {
        const double t = cs[i] * col[i] + sn[i] * col[i + 1];
        col[i + 1] = -sn[i] * col[i] + cs[i] * col[i + 1];
        col[i] = t;
      }
      const double d = std::hypot(col[j], col[j + 1]);
      cs[j] = d > 0.0 ? col[j] / d : 1.0;
      sn[j] = d > 0.0 ? col[j + 1] / d : 0.0;
      col[j] = d;
      col[j + 1] = 0.0;
      g[j + 1] = -sn[j] * g[j];
      g[j] = cs[j] * g[j];
      for (int i = 0; i <= j; ++i) H[(size_t)i * m + j] = col[i];
      ++j;
      ++total;
      rel = std::fabs(g[j]) / scale;
      if (!std::isfinite(rel) || rel < tol || !(hn > 0.0)) break;
    }
    // x += Z y with R y = g (R: the rotated Hessenberg, upper triangular)
    for (int i = j - 1; i >= 0; --i) {
      double t = g[i];
      for (int k = i + 1; k < j; ++k) t -= H[(size_t)i * m + k] * y[k];
      y[i] = H[(size_t)i * m + i] != 0.0 ? t / H[(size_t)i * m + i] : 0.0;
    }
    std::copy(y.begin(), y.begin() + j, h->gmHost);
    GB_CUDA(h, cudaMemcpyAsync(h->gmDev, h->gmHost, j * sizeof(double), cudaMemcpyHostToDevice, s));
    LAUNCH(h, VC, launch_maxpy(s, h->p, h->gmZ, n, h->gmDev, j, 1.0, n));
    f.sol = h->p; f.src = h->b;
    LAUNCH(h, GBMG_PROF_RESIDUAL,
           launch_residual_norm<double>(s, v64(f), h->kr, h->red, kSlotNorm));
    GB_TRY(check_launch(h, "fgmres residual"));
    GB_TRY(read_result(h, kSlotNorm, &r2));
    rel = std::sqrt(r2) / scale;
    if (!std::isfinite(rel) || rel > 1e3) { *status = GBMG_DIVERGED; break; }
    if (rel < tol) { *status = GBMG_OK; break; }
  }
  *rel_io = rel;
  *cycles = total;
  return GBMG_OK;
}

// Start of the stationary mixed loop.  A zero initial p goes straight into
// the double-word pressure.  A warm start (p != 0) is solved as a correction:
// r0 = b - A p in native FP64 becomes the loop's right-hand side and the loop
// solves A d = r0 from d = 0; finish_mixed then adds d to p in FP64.  The
// double-word operator rounds relative to |A||p|, and for a warm start |b| can
// be far below |A||p| (a later pass of a time step), which would put the loop's
// floor near the tolerance; in the correction form it rounds relative to
// |A||d| instead.  *shifted tells finish_mixed which form ran.
int start_mixed(gbmg_handle* h, bool* shifted) {
  const cudaStream_t s = h->stream;
  Level& f = h->lv[0];
  const size_t n = h->n0;
  if (h->p_nonzero >= 0) {
    // tested with the right-hand side
    *shifted = h->p_nonzero != 0;
    h->p_nonzero = -1;
  } else {
    LAUNCH(h, GBMG_PROF_VECTOR, launch_nonzero(s, h->p, n, h->red.result + kSlotSum + 1));
    GB_TRY(check_launch(h, "initial guess"));
    double pp = 0.0;
    GB_TRY(read_result(h, kSlotSum + 1, &pp));
    unsigned long long nz = 0ull;
    std::memcpy(&nz, &pp, sizeof(nz));
    *shifted = nz != 0ull;
  }
  if (*shifted) {
    // the correction starts at d = 0, so its first residual is r0 itself:
    // the loop's right-hand side in double-word and the FP32 cycle's input
    if (!h->r0) GB_TRY(dmalloc(h, &h->r0, n));
    f.sol = h->p; f.src = h->b;
    LAUNCH(h, GBMG_PROF_RESIDUAL, launch_residual_norm<double>(s, v64(f), h->r0, h->red, kSlotNorm));
    LAUNCH(h, GBMG_PROF_VECTOR, launch_to_dw(s, h->r0, h->bw, n));
    if (f.split) LAUNCH(h, GBMG_PROF_VECTOR, launch_to_split(s, h->r0, f.src32, f.nx, f.ny, f.nz, f.hstride));
    else LAUNCH(h, GBMG_PROF_VECTOR, launch_double_to_float(s, h->r0, f.src32, n));
    GB_CUDA(h, cudaMemsetAsync(h->pw[1], 0, n * sizeof(float2), s));
  } else {
    // p = 0: the first residual is b.  The right-hand side's preparation
    // already wrote its FP32 copy, b rounded to float (what the defect kernel
    // would store: the double-word b's hi is b rounded to nearest, and
    // hi + lo rounds back to it), and its norm; the double-word p is zero.
    GB_CUDA(h, cudaMemsetAsync(h->pw[1], 0, n * sizeof(float2), s));
    GB_CUDA(h, cudaMemcpyAsync(h->red.result + kSlotNorm, h->red.result + kSlotSumB + 1,
                               sizeof(double), cudaMemcpyDeviceToDevice, s));
  }
  h->pcur = 1;
  return GBMG_OK;
}

// The mixed loop's result into h->p, mean-free (compatibility_sol on the
// finest level).  After a correction solve the double-word right-hand side
// still holds r0; every solve writes it afresh before its loop.
int finish_mixed(gbmg_handle* h, bool shifted) {
  const cudaStream_t s = h->stream;
  const size_t n = h->n0;
  if (shifted) {
    LAUNCH(h, GBMG_PROF_VECTOR, launch_dw_accumulate(s, h->pw[h->pcur], h->p, n));
    LAUNCH(h, GBMG_PROF_VECTOR, launch_sum(s, h->p, n, h->red, kSlotSum));
    LAUNCH(h, GBMG_PROF_VECTOR, launch_shift_by_mean(s, h->p, h->p, n, h->red, kSlotSum, -1));
  } else {
    LAUNCH(h, GBMG_PROF_VECTOR, launch_dw_sum(s, h->pw[h->pcur], n, h->red, kSlotSum));
    LAUNCH(h, GBMG_PROF_VECTOR, launch_dw_out(s, h->pw[h->pcur], h->p, n, h->red, kSlotSum));
  }
  return check_launch(h, "mean");
}

// Restarts of the stationary mixed loop after a failed FP64 certification.
constexpr int kMixedRestarts = 2;

int solve_internal(gbmg_handle* h, double tol, double bnorm, gbmg_stats* st) {
  const cudaStream_t s = h->stream;
  Level& f = h->lv[0];
  const size_t n = h->n0;
  const bool pcg = h->prm.krylov != 0;
  const int kind = pcg ? (h->mixed ? kGraphPcgMixed : kGraphPcg64) : (h->mixed ? kGraphMixed : kGraphFp64);
  const double scale = bnorm > 0.0 ? bnorm : 1.0;
  // Stopping rules.  RMS: sqrt(|r|^2/n) < tol is |r|/|b| < tol sqrt(n)/|b|, so
  // the relative test below runs with that threshold.  INCREMENT: the loop
  // stops on max |p_k - p_(k-1)| < tol; the residual is only reported.
  const bool by_inc = h->prm.stop_rule == GBMG_STOP_INCREMENT;
  if (h->prm.stop_rule == GBMG_STOP_RMS) tol = tol * std::sqrt((double)n) / scale;
  const double rtol = by_inc ? 0.0 : tol;  // threshold of the residual tests
  bool shifted = false;
  // initial residual
  f.sol = h->p; f.src = h->b;
  if (pcg) {
    LAUNCH(h, GBMG_PROF_RESIDUAL, launch_residual_norm<double>(s, v64(f), h->kr, h->red, kSlotNorm));
    GB_CUDA(h, cudaMemsetAsync(h->kzold, 0, n * sizeof(double), s));
  } else if (h->mixed) {
    GB_TRY(start_mixed(h, &shifted));
  } else {
    LAUNCH(h, GBMG_PROF_RESIDUAL,
           launch_residual_norm<double>(s, v64(f), (double*)nullptr, h->red, kSlotNorm));
  }
  GB_TRY(check_launch(h, "residual"));
  double r2 = 0.0;
  GB_TRY(read_result(h, kSlotNorm, &r2));
  double rel = std::sqrt(r2) / scale;
  st->res0 = rel;
  int status = GBMG_NOT_CONVERGED;
  int cyc = 0;
  if (rel < rtol || r2 == 0.0) {
    status = GBMG_OK;
  } else if (h->prm.krylov == 2) {
    GB_TRY(fgmres(h, tol, scale, &rel, &cyc, &status));
    r2 = rel * scale * rel * scale;
  }
  for (int restart = 0;; ++restart) {
    bool stalled = false;  // the mixed loop stopped on a flat tracked residual
    if (status == GBMG_NOT_CONVERGED && h->prm.krylov != 2) {
      double best = rel;
      int flat = 0;
      // cycles of the next iteration (the adaptive mixed loop shortens the
      // last correction to what tail_cycles predicts)
      const bool adapt = kind == kGraphMixed && h->adaptive && !h->stag_mode;
      int next = kind == kGraphMixed ? (h->stag_mode ? 1 : h->inner) : 1;
      while (cyc < h->prm.max_cycles) {
        // every iteration of full length but the first flexible-CG one: the
        // loop on the device
        if (!(pcg && cyc == 0) && next == (kind == kGraphMixed ? h->inner : 1)) {
          CycleCtl c{};
          c.scale = scale;
          c.tol = tol;
          c.guard = 1e3 * std::max(1.0, st->res0);
          c.best = best;
          c.max_cycles = h->prm.max_cycles;
          c.step = kind == kGraphMixed ? h->inner : 1;
          c.by_inc = by_inc ? 1 : 0;
          c.flat_stop = (kind == kGraphMixed && h->prm.certify) ? 1 : 0;
          c.cyc = cyc;
          c.flat = flat;
          c.rel = rel;
          c.adaptive = adapt ? 1 : 0;
          bool used = false;
          GB_TRY(run_loop(h, kind, &c, &used));
          if (used) {
            if (kind == kGraphMixed) h->pcur ^= c.iters & 1;
            st->device_loop = 1;
            if (c.iters > 0) {
              cyc = c.cyc;
              r2 = c.r2;
              rel = c.rel;
              best = c.best;
              flat = c.flat;
              if (by_inc) st->increment = c.inc;
              if (c.status == kCtlDiverged) status = GBMG_DIVERGED;
              else if (c.status == kCtlConverged) status = GBMG_OK;
              stalled = c.stalled != 0;
            }
            // ended by a test, by the predicted last correction (run below),
            // or with too few cycles left for a whole iteration (run below)
            if (status != GBMG_NOT_CONVERGED || stalled || cyc >= h->prm.max_cycles) break;
            if (c.tail > 0) next = c.tail;
          }
        }
        const int step = kind == kGraphMixed ? std::min(next, h->prm.max_cycles - cyc) : 1;
        const double prev = rel;
        cyc += step;
        GB_TRY(run_iteration(h, kind, pcg && cyc == 1, step));
        if (kind == kGraphMixed) h->pcur ^= 1;
        GB_CUDA(h, cudaStreamSynchronize(s));
        prof_flush(h);
        r2 = h->host_res[kSlotNorm];
        rel = std::sqrt(r2) / scale;
        if (!std::isfinite(rel) || rel > 1e3 * std::max(1.0, st->res0)) {
          status = GBMG_DIVERGED;
          break;
        }
        if (h->stag_mode) {
          // the split driver's test: a cycle that does not cut the residual
          // by 1% (or raises it) stagnates
          const double grow = rel / prev;
          if (grow > 1.0 || std::fabs(grow - 1.0) < 0.01) {
            if (h->stag_mode == 1) {
              h->stagnated = true;
              break;
            }
            if (rel < 1000.0 * tol) { status = GBMG_OK; break; }
          } else if (rel < tol) {
            status = GBMG_OK;
            break;
          }
          continue;
        }
        if (by_inc) {
          double dp = 0.0;
          std::memcpy(&dp, &h->host_res[kSlotInc], sizeof(double));
          st->increment = dp;
          if (dp < tol) { status = GBMG_OK; break; }
          continue;
        }
        if (rel < tol) { status = GBMG_OK; break; }
        if (adapt) next = tail_cycles(rel, prev, tol, step, h->inner);
        // The mixed cycle tracks its residual in double-word FP32; near the
        // tolerance that figure can level off while the FP64 residual is
        // already below it.  Four cycles without any decrease end the loop and
        // leave the decision to the FP64 certification below.
        if (kind == kGraphMixed && h->prm.certify) {
          if (rel < best) {
            best = rel;
            flat = 0;
          } else if (++flat >= 4) {
            stalled = true;
            break;
          }
        }
      }
    }
    // mean projection of p (compatibility_sol on the finest level)
    if (kind == kGraphMixed) {
      GB_TRY(finish_mixed(h, shifted));
    } else {
      LAUNCH(h, GBMG_PROF_VECTOR, launch_sum(s, h->p, n, h->red, kSlotSum));
      LAUNCH(h, GBMG_PROF_VECTOR, launch_shift_by_mean(s, h->p, h->p, n, h->red, kSlotSum, -1));
      GB_TRY(check_launch(h, "mean"));
    }
    if (h->dl_field) {
      // p is final unless the certification below sends the loop round again:
      // its copy to the host runs beside the certification
      GB_CUDA(h, cudaEventRecord(h->cev[1], s));
      GB_CUDA(h, cudaStreamWaitEvent(h->cstream, h->cev[1], 0));
      GB_TRY(download(h, h->p, h->grid.nx, h->grid.ny, h->grid.nz, GBMG_MEM_HOST, *h->dl_field,
                      h->cstream));
      h->dl_started = true;
    }
    if (!(kind == kGraphMixed && h->prm.certify)) break;
    if (h->stagnated) {  // the caller restarts; report the FP64 residual
      f.sol = h->p; f.src = h->b;
      LAUNCH(h, GBMG_PROF_CERTIFY,
             launch_residual_norm<double>(s, v64(f), (double*)nullptr, h->red, kSlotNorm));
      GB_TRY(check_launch(h, "certify"));
      GB_TRY(read_result(h, kSlotNorm, &r2));
      rel = std::sqrt(r2) / scale;
      break;
    }
    if (by_inc) {
      // reported only: the increment decided
      f.sol = h->p; f.src = h->b;
      LAUNCH(h, GBMG_PROF_CERTIFY,
             launch_residual_norm<double>(s, v64(f), (double*)nullptr, h->red, kSlotNorm));
      GB_TRY(check_launch(h, "certify"));
      GB_TRY(read_result(h, kSlotNorm, &r2));
      rel = std::sqrt(r2) / scale;
      break;
    }
    // the loop tracked the residual in double-word; restate it in native FP64
    f.sol = h->p; f.src = h->b;
    LAUNCH(h, GBMG_PROF_CERTIFY,
           launch_residual_norm<double>(s, v64(f), (double*)nullptr, h->red, kSlotNorm));
    GB_TRY(check_launch(h, "certify"));
    GB_TRY(read_result(h, kSlotNorm, &r2));
    rel = std::sqrt(r2) / scale;
    if (status == GBMG_OK && !(rel < tol)) status = GBMG_NOT_CONVERGED;
    if (status == GBMG_NOT_CONVERGED && stalled && rel < tol) status = GBMG_OK;
    if (status != GBMG_NOT_CONVERGED || cyc >= h->prm.max_cycles || restart >= kMixedRestarts)
      break;
    // Certified above the tolerance with cycles left: go round again from the
    // certified p, as a correction solve (its residual is the FP64 one just
    // computed).  The host copy started above must finish before p changes.
    if (h->dl_field) {
      GB_CUDA(h, cudaEventRecord(h->cev[0], h->cstream));
      GB_CUDA(h, cudaStreamWaitEvent(s, h->cev[0], 0));
    }
    GB_TRY(start_mixed(h, &shifted));
    GB_TRY(read_result(h, kSlotNorm, &r2));
    rel = std::sqrt(r2) / scale;
    if (rel < tol) status = GBMG_OK;
  }
  {
    // the flag came back with the last results when no kernel ran since
    int flags = 0;
    if (h->flags_at == h->launches) {
      std::memcpy(&flags, h->host_res + kRedSlots, sizeof(int));
    } else {
      GB_CUDA(h, cudaMemcpyAsync(&flags, h->derr, sizeof(int), cudaMemcpyDeviceToHost, s));
      GB_CUDA(h, cudaStreamSynchronize(s));
    }
    if (flags) {
      h->err = "a bulk-copy wait timed out inside a kernel of the cycle";
      cudaMemsetAsync(h->derr, 0, sizeof(int), s);
      return GBMG_CUDA_ERROR;
    }
  }
  st->status = status;
  st->cycles = cyc;
  st->levels = h->L;
  st->coarse_n = h->nc;
  st->rel_residual = rel;
  st->rms_residual = std::sqrt(r2 / (double)n);
  // algorithmic bytes per cycle: the V-cycle, plus the residual of each
  // iteration (FP64: p, b, cx, cy, cz; or the defect with its e read, p write,
  // r32 write and zeroed e)
  const int w = h->mixed ? 4 : 8;
  double per = vcycle_bytes(h, w);
  if (kind == kGraphMixed) per += (40.0 * n + 16.0 * n + 4.0 * n) / h->inner;
  else per += 40.0 * n + (h->mixed ? 20.0 * n : 0.0);
  if (pcg) per += (h->mixed ? 24.0 : 8.0) * n + 16.0 * n + 32.0 * n + 48.0 * n + 24.0 * n + 8.0 * n;
  st->bytes = per * cyc + 40.0 * n + 32.0 * n;
  return status;
}


// Face velocities on the device: the caller's arrays (device memory) or
// staging copies of them (host memory).
int stage_velocity(gbmg_handle* h, const gbmg_field* const fv[3], bool has_w, int mem,
                   double* dv[3], gbmg_field dfield[3]) {
  const gbmg_grid& g = h->grid;
  const int ext[3][3] = {{g.nx + 1, g.ny, g.nz}, {g.nx, g.ny + 1, g.nz}, {g.nx, g.ny, g.nz + 1}};
  for (int a = 0; a < 3; ++a) {
    if (a == 2 && !has_w) continue;
    const size_t n = (size_t)ext[a][0] * ext[a][1] * ext[a][2];
    if (mem == GBMG_MEM_DEVICE) {
      dv[a] = fv[a]->data;
      dfield[a] = *fv[a];
    } else {
      if (h->vel_n[a] < n) {
        dfree(h->vel[a]);
        GB_TRY(dmalloc(h, &h->vel[a], n));
        h->vel_n[a] = n;
      }
      GB_TRY(upload(h, *fv[a], ext[a][0], ext[a][1], ext[a][2], mem, h->vel[a]));
      dv[a] = h->vel[a];
      dfield[a] = gbmg_field{h->vel[a], ext[a][0], (int64_t)ext[a][0] * ext[a][1]};
    }
  }
  return GBMG_OK;
}

// RHSP's wall-normal faces set to zero on the device copies of u, v, w
// (gbmg_params.zero_wall_faces; nothing otherwise).
int zero_walls(gbmg_handle* h, const gbmg_field dfield[3], bool has_w) {
  if (!h->prm.zero_wall_faces) return GBMG_OK;
  const gbmg_grid& g = h->grid;
  launch_zero_wall_faces(h->stream, g.nx, g.ny, g.nz, dfield[0].data, dfield[0].sy, dfield[0].sz,
                         dfield[1].data, dfield[1].sy, dfield[1].sz,
                         has_w ? dfield[2].data : nullptr, has_w ? dfield[2].sy : 0,
                         has_w ? dfield[2].sz : 0);
  h->launches += 1;
  return check_launch(h, "zero_wall_faces");
}

}  // namespace

namespace gbmg {
namespace host {

// The projection on device face velocities (fields addressed at their face
// (0,0,0)) with the initial pressure already in h->p: b = div(u*)/dt, the
// solve, then u -= dt beta grad p (ppe_sor_solver + ns_momentum_correction).
int project_device(gbmg_handle* h, const gbmg_field dfield[3], bool has_w, double dt, double tol,
                   gbmg_stats* st) {
  const gbmg_grid& g = h->grid;
  const cudaStream_t s = h->stream;
  Strided su{dfield[0].data, dfield[0].sy, dfield[0].sz};
  Strided sv{dfield[1].data, dfield[1].sy, dfield[1].sz};
  Strided sw{has_w ? dfield[2].data : nullptr, has_w ? dfield[2].sy : 0,
             has_w ? dfield[2].sz : 0};
  GB_TRY(zero_walls(h, dfield, has_w));
  launch_divergence(s, g.nx, g.ny, g.nz, su, sv, sw, g.dx, g.dy, g.dz, dt, h->b);
  h->launches += 1;
  GB_TRY(check_launch(h, "divergence"));
  // mean projection + norm of b in place
  double bnorm = 0.0;
  GB_TRY(finish_rhs(h, &bnorm));
  const int status = solve_internal(h, tol, bnorm, st);
  if (status != GBMG_OK && status != GBMG_NOT_CONVERGED && status != GBMG_DIVERGED) return status;
  launch_correct(s, g.nx, g.ny, g.nz, h->rho, h->p, g.dx, g.dy, g.dz, dt, dfield[0].data,
                 dfield[0].sy, dfield[0].sz, dfield[1].data, dfield[1].sy, dfield[1].sz,
                 has_w ? dfield[2].data : nullptr, has_w ? dfield[2].sy : 0,
                 has_w ? dfield[2].sz : 0);
  h->launches += 1;
  GB_TRY(check_launch(h, "correct"));
  return status;
}

}  // namespace host
}  // namespace gbmg


// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" {

void gbmg_default_params(gbmg_params* prm) {
  if (!prm) return;
  std::memset(prm, 0, sizeof(*prm));
  prm->precision = GBMG_PREC_FP64;
  prm->nu1 = 2;
  prm->nu2 = 2;
  prm->levels = 0;
  prm->coarse_max = 64;
  prm->max_cycles = 100;
  prm->krylov = 0;
  prm->use_graph = 1;
  prm->remove_rhs_mean = 1;
  prm->certify = 1;
  prm->device = -1;
  prm->stream = nullptr;
}

int gbmg_create(const gbmg_grid* grid, const gbmg_params* prm, gbmg_handle** out) {
  if (!grid || !out) return GBMG_INVALID_ARG;
  *out = nullptr;
  if (grid->nx < 1 || grid->ny < 1 || grid->nz < 1 || !(grid->dx > 0) || !(grid->dy > 0) ||
      (grid->nz > 1 && !(grid->dz > 0)))
    return GBMG_INVALID_ARG;
  // the parameters are checked before any CUDA call
  gbmg_params P;
  if (prm) P = *prm; else gbmg_default_params(&P);
  if (P.nu1 < 0 || P.nu2 < 0 || P.max_cycles < 1 || P.coarse_max < 1 ||
      P.coarse_max > kMaxCoarse ||
      (P.precision != GBMG_PREC_FP64 && P.precision != GBMG_PREC_MIXED) ||
      P.stop_rule < GBMG_STOP_RELATIVE || P.stop_rule > GBMG_STOP_INCREMENT ||
      (P.stop_rule == GBMG_STOP_INCREMENT && P.krylov != 0) ||
      (P.zero_wall_faces != 0 && P.zero_wall_faces != 1) || P.use_graph < 0 ||
      P.use_graph > 2 || P.inner_cycles < 0 || P.inner_cycles > 8 || P.split_restarts < 0 ||
      P.split_restarts > 100 || (P.split_restarts > 0 && P.krylov != 0) ||
      (P.inner_cycles > 1 && P.stop_rule == GBMG_STOP_INCREMENT))
    return GBMG_INVALID_ARG;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
    cudaGetLastError();
    return GBMG_NO_DEVICE;
  }
  gbmg_handle* h = new gbmg_handle();
  h->grid = *grid;
  if (h->grid.nz == 1 && !(h->grid.dz > 0)) h->grid.dz = 1.0;
  h->prm = P;
  h->mixed = h->prm.precision == GBMG_PREC_MIXED;
  // Several FP32 cycles per defect correction: the FP32 correction is good to
  // about 1e-6 of its size, so later cycles still gain their full factor,
  // and defect kernels are saved.  By default four per correction while the
  // residual is far from the tolerance (five left a warm start far from its
  // solution above 1e-10), then as many as tail_cycles predicts, so that the
  // cycle count stays the per-cycle test's.  The increment rule measures one
  // cycle.
  h->adaptive = h->prm.inner_cycles == 0 && h->prm.stop_rule != GBMG_STOP_INCREMENT;
  h->inner = h->prm.inner_cycles > 0 ? h->prm.inner_cycles : (h->adaptive ? 4 : 1);
  if (h->prm.device >= 0) {
    if (h->prm.device >= ndev) { delete h; return GBMG_INVALID_ARG; }
    h->device = h->prm.device;
  } else {
    cudaGetDevice(&h->device);
  }
  if (cudaSetDevice(h->device) != cudaSuccess) { delete h; return GBMG_CUDA_ERROR; }
  if (h->prm.stream) {
    h->stream = (cudaStream_t)h->prm.stream;
    h->own_stream = false;
  } else {
    if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess) {
      delete h;
      return GBMG_CUDA_ERROR;
    }
    h->own_stream = true;
  }
  const int rc = allocate(h);
  if (rc != GBMG_OK) {
    std::fprintf(stderr, "gbmg_create: %s\n", h->err.c_str());
    free_all(h);
    delete h;
    return rc;
  }
  *out = h;
  return GBMG_OK;
}

int gbmg_destroy(gbmg_handle* h) {
  if (!h) return GBMG_INVALID_ARG;
  cudaSetDevice(h->device);
  if (h->stream) cudaStreamSynchronize(h->stream);
  free_all(h);
  delete h;
  return GBMG_OK;
}

int gbmg_set_rho(gbmg_handle* h, gbmg_field rho, int mem) {
  GB_TRY(begin(h));
  GB_TRY(validate_field(h, rho, "rho"));
  const gbmg_grid& g = h->grid;
  GB_TRY(upload(h, rho, g.nx, g.ny, g.nz, mem, h->rho));
  GB_CUDA(h, cudaEventRecord(h->cev[4], h->stream));
  GB_TRY(set_rho_device(h, nullptr));
  // The set-up kernels run on after the call returns (the next call on the
  // handle is ordered after them on its stream); the caller's rho has been
  // read once the copy is done.
  GB_CUDA(h, cudaEventSynchronize(h->cev[4]));
  return GBMG_OK;
}

int gbmg_set_phi(gbmg_handle* h, gbmg_field phi, double eps, double rho_pos, double rho_neg,
                 int mem) {
  GB_TRY(begin(h));
  GB_TRY(validate_field(h, phi, "phi"));
  if (!(eps > 0)) { h->err = "eps must be > 0"; return GBMG_INVALID_ARG; }
  const gbmg_grid& g = h->grid;
  const double* src = phi.data;
  Strided sp{phi.data, phi.sy, phi.sz};
  if (mem == GBMG_MEM_HOST) {
    GB_TRY(upload(h, phi, g.nx, g.ny, g.nz, mem, h->p));  // p as staging
    sp = Strided{h->p, g.nx, (int64_t)g.nx * g.ny};
  }
  (void)src;
  launch_rho_from_phi(h->stream, g.nx, g.ny, g.nz, sp, eps, rho_pos, rho_neg, h->rho);
  h->launches += 1;
  GB_TRY(check_launch(h, "rho_from_phi"));
  // phi (and the staging copy in p) has been read by here
  GB_CUDA(h, cudaEventRecord(h->cev[3], h->stream));
  // away from the interface rho is exactly rho_pos*1 + rho_neg*0 or rho_pos*0 + rho_neg*1
  const double bulk[2] = {rho_pos * 1.0 + rho_neg * (1.0 - 1.0), rho_pos * 0.0 + rho_neg * (1.0 - 0.0)};
  GB_TRY(set_rho_device(h, bulk));
  // The remaining set-up kernels run on after the call returns (the next call
  // on the handle is ordered after them on its stream; a solve from host
  // arrays uploads b and p beside them).
  GB_CUDA(h, cudaEventSynchronize(h->cev[3]));
  return GBMG_OK;
}

int gbmg_set_coef(gbmg_handle* h, gbmg_field cx, gbmg_field cy, gbmg_field cz, int mem) {
  GB_TRY(begin(h));
  GB_TRY(validate_field(h, cx, "cx"));
  GB_TRY(validate_field(h, cy, "cy"));
  GB_TRY(validate_field(h, cz, "cz"));
  const gbmg_grid& g = h->grid;
  Level& f = h->lv[0];
  GB_TRY(upload(h, cx, g.nx, g.ny, g.nz, mem, f.cx));
  GB_TRY(upload(h, cy, g.nx, g.ny, g.nz, mem, f.cy));
  GB_TRY(upload(h, cz, g.nx, g.ny, g.nz, mem, f.cz));
  // the wall entries are taken as walls whatever the caller stored there
  for (int k = 0; k < g.nz; ++k) {
    GB_CUDA(h, cudaMemset2DAsync(f.cx + (size_t)k * g.nx * g.ny, (size_t)g.nx * sizeof(double), 0,
                                 sizeof(double), (size_t)g.ny, h->stream));
  }
  GB_CUDA(h, cudaMemsetAsync(f.cz, 0, (size_t)g.nx * g.ny * sizeof(double), h->stream));
  for (int k = 0; k < g.nz; ++k)
    GB_CUDA(h, cudaMemsetAsync(f.cy + (size_t)k * g.nx * g.ny, 0, (size_t)g.nx * sizeof(double),
                               h->stream));
  h->rho_ready = false;
  h->split_ready = false;
  h->fine_copies = false;
  set_rho_form(h, false);
  GB_TRY(build_hierarchy(h));
  GB_CUDA(h, cudaStreamSynchronize(h->stream));
  return GBMG_OK;
}

int gbmg_solve(gbmg_handle* h, gbmg_field b, gbmg_field p, double tol, int mem,
               gbmg_stats* stats) {
  GB_TRY(begin(h));
  gbmg_stats local{};
  gbmg_stats* st = stats ? stats : &local;
  std::memset(st, 0, sizeof(*st));
  if (!h->coef_ready) { h->err = "no coefficients: call gbmg_set_rho/phi/coef first"; return GBMG_STATE_ERROR; }
  GB_TRY(validate_field(h, b, "b"));
  GB_TRY(validate_field(h, p, "p"));
  if (!(tol > 0)) { h->err = "tol must be > 0"; return GBMG_INVALID_ARG; }
  const gbmg_grid& g = h->grid;
  GB_CUDA(h, cudaEventRecord(h->ev0, h->stream));
  double bnorm = 0.0;
  const bool host = mem == GBMG_MEM_HOST;
  if (host) {
    // host memory: b and the initial p cross to the device on the handle's
    // second stream, beside the operator set-up still running from
    // gbmg_set_phi / gbmg_set_rho (which reads neither b nor p once the
    // staging copy in p has been consumed: cev[3]) and beside the right-hand
    // side's preparation; the result crosses back beside the certification
    GB_CUDA(h, cudaStreamWaitEvent(h->cstream, h->cev[3], 0));
    GB_TRY(upload(h, b, g.nx, g.ny, g.nz, mem, h->b, h->cstream));
    GB_CUDA(h, cudaEventRecord(h->cev[2], h->cstream));
    GB_TRY(upload(h, p, g.nx, g.ny, g.nz, mem, h->p, h->cstream));
    GB_CUDA(h, cudaEventRecord(h->cev[0], h->cstream));
    GB_CUDA(h, cudaStreamWaitEvent(h->stream, h->cev[2], 0));
    const int rc = finish_rhs(h, &bnorm, true, h->cev[0]);
    if (rc != GBMG_OK) {
      cudaStreamSynchronize(h->cstream);  // the caller's p may be freed on return
      return rc;
    }
    GB_CUDA(h, cudaStreamWaitEvent(h->stream, h->cev[0], 0));
  } else {
    GB_TRY(upload(h, b, g.nx, g.ny, g.nz, mem, h->b));
    GB_TRY(upload(h, p, g.nx, g.ny, g.nz, mem, h->p));
    GB_TRY(finish_rhs(h, &bnorm, true));
  }
  h->dl_field = host ? &p : nullptr;
  h->dl_started = false;
  const int status = solve_internal(h, tol, bnorm, st);
  h->dl_field = nullptr;
  const bool downloaded = h->dl_started;
  if (h->dl_started) {
    h->dl_started = false;
    GB_CUDA(h, cudaEventRecord(h->cev[0], h->cstream));
    GB_CUDA(h, cudaStreamWaitEvent(h->stream, h->cev[0], 0));
  }
  if (status != GBMG_OK && status != GBMG_NOT_CONVERGED && status != GBMG_DIVERGED) {
    cudaStreamSynchronize(h->cstream);
    return status;
  }
  if (!host) GB_TRY(download(h, h->p, g.nx, g.ny, g.nz, mem, p));
  else if (!downloaded) GB_TRY(download(h, h->p, g.nx, g.ny, g.nz, mem, p));
  GB_CUDA(h, cudaEventRecord(h->ev1, h->stream));
  GB_CUDA(h, cudaEventSynchronize(h->ev1));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, h->ev0, h->ev1);
  st->ms = ms;
  st->bytes += 16.0 * h->n0;
  return status;
}

int gbmg_project(gbmg_handle* h, gbmg_field u, gbmg_field v, gbmg_field w, gbmg_field p,
                 double dt, double tol, int mem, gbmg_stats* stats) {
  GB_TRY(begin(h));
  gbmg_stats local{};
  gbmg_stats* st = stats ? stats : &local;
  std::memset(st, 0, sizeof(*st));
  if (!h->coef_ready || !h->rho_ready) {
    h->err = "the projection needs the density: call gbmg_set_rho or gbmg_set_phi first";
    return GBMG_STATE_ERROR;
  }
  GB_TRY(validate_field(h, u, "u"));
  GB_TRY(validate_field(h, v, "v"));
  GB_TRY(validate_field(h, p, "p"));
  const bool has_w = w.data != nullptr && h->grid.nz > 1;
  if (has_w) GB_TRY(validate_field(h, w, "w"));
  if (!(dt > 0) || !(tol > 0)) { h->err = "dt and tol must be > 0"; return GBMG_INVALID_ARG; }
  const gbmg_grid& g = h->grid;
  const cudaStream_t s = h->stream;
  GB_CUDA(h, cudaEventRecord(h->ev0, s));
  const int ext[3][3] = {{g.nx + 1, g.ny, g.nz}, {g.nx, g.ny + 1, g.nz}, {g.nx, g.ny, g.nz + 1}};
  const gbmg_field* fv[3] = {&u, &v, &w};
  double* dv[3] = {nullptr, nullptr, nullptr};
  gbmg_field dfield[3];
  GB_TRY(stage_velocity(h, fv, has_w, mem, dv, dfield));
  GB_TRY(upload(h, p, g.nx, g.ny, g.nz, mem, h->p));
  const int status = project_device(h, dfield, has_w, dt, tol, st);
  if (status != GBMG_OK && status != GBMG_NOT_CONVERGED && status != GBMG_DIVERGED) return status;
  if (mem == GBMG_MEM_HOST)
    for (int a = 0; a < 3; ++a) {
      if (a == 2 && !has_w) continue;
      GB_TRY(download(h, dv[a], ext[a][0], ext[a][1], ext[a][2], mem, *fv[a]));
    }
  GB_TRY(download(h, h->p, g.nx, g.ny, g.nz, mem, p));
  GB_CUDA(h, cudaEventRecord(h->ev1, s));
  GB_CUDA(h, cudaEventSynchronize(h->ev1));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, h->ev0, h->ev1);
  st->ms = ms;
  return status;
}

int gbmg_set_split(gbmg_handle* h, gbmg_field rho, double rho_12, int mem) {
  GB_TRY(begin(h));
  GB_TRY(validate_field(h, rho, "rho"));
  if (!(rho_12 > 0)) { h->err = "rho_12 must be > 0"; return GBMG_INVALID_ARG; }
  const gbmg_grid& g = h->grid;
  GB_TRY(upload(h, rho, g.nx, g.ny, g.nz, mem, h->rho));
  Level& f = h->lv[0];
  float* c32[3] = {f.cx32, f.cy32, f.cz32};
  float2* cw[3] = {h->cxw, h->cyw, h->czw};
  LAUNCH(h, GBMG_PROF_SETUP,
         launch_face_const(h->stream, g.nx, g.ny, g.nz, g.dx * g.dx, g.dy * g.dy, g.dz * g.dz, f.cx,
                           f.cy, f.cz, h->mixed ? c32 : nullptr, h->mixed ? cw : nullptr));
  GB_TRY(check_launch(h, "face_const"));
  h->fine_copies = h->mixed;
  set_rho_form(h, false);
  h->rho_ready = false;  // the operator is not the density's: no plain projection or adjoint
  GB_TRY(build_hierarchy(h));
  h->split_ready = true;
  h->split_rho12 = rho_12;
  GB_CUDA(h, cudaStreamSynchronize(h->stream));
  return GBMG_OK;
}

int gbmg_project_split(gbmg_handle* h, gbmg_field u, gbmg_field v, gbmg_field w,
                       gbmg_field p_hat, gbmg_field p, double dt, double tol, int mem,
                       gbmg_stats* stats) {
  GB_TRY(begin(h));
  gbmg_stats local{};
  gbmg_stats* st = stats ? stats : &local;
  std::memset(st, 0, sizeof(*st));
  if (!h->split_ready || !h->coef_ready) {
    h->err = "the split projection needs gbmg_set_split first";
    return GBMG_STATE_ERROR;
  }
  GB_TRY(validate_field(h, u, "u"));
  GB_TRY(validate_field(h, v, "v"));
  GB_TRY(validate_field(h, p_hat, "p_hat"));
  GB_TRY(validate_field(h, p, "p"));
  const bool has_w = h->grid.nz > 1;
  if (has_w) GB_TRY(validate_field(h, w, "w"));
  if (!(dt > 0) || !(tol > 0)) { h->err = "dt and tol must be > 0"; return GBMG_INVALID_ARG; }
  const gbmg_grid& g = h->grid;
  const cudaStream_t s = h->stream;
  GB_CUDA(h, cudaEventRecord(h->ev0, s));
  const gbmg_field* fv[3] = {&u, &v, &w};
  double* dv[3] = {nullptr, nullptr, nullptr};
  gbmg_field dfield[3];
  GB_TRY(stage_velocity(h, fv, has_w, mem, dv, dfield));
  // p^ into aux[0]; the solve starts from it (the reference's mg sol = p%tmp)
  if (!h->aux[0]) GB_TRY(dmalloc(h, &h->aux[0], h->n0));
  GB_TRY(upload(h, p_hat, g.nx, g.ny, g.nz, mem, h->aux[0]));
  Strided su{dv[0], dfield[0].sy, dfield[0].sz}, sv{dv[1], dfield[1].sy, dfield[1].sz};
  Strided sw{has_w ? dv[2] : nullptr, has_w ? dfield[2].sy : 0, has_w ? dfield[2].sz : 0};
  GB_TRY(zero_walls(h, dfield, has_w));
  // The driver's restarts: a stagnating cycle ends the solve, p^ becomes
  // 1.5 p - 0.5 p^ and the source is rebuilt from it
  // ("DomainDecomposition/3D/src/ns_solver/ns_ppe_mg_solver.f90:29-44").
  const int nres = h->prm.split_restarts;
  int status = GBMG_OK, cycles = 0, restart = 0;
  for (;; ++restart) {
    launch_psplit_rhs(s, g.nx, g.ny, g.nz, h->rho, su, sv, sw, h->aux[0], h->split_rho12, g.dx,
                      g.dy, g.dz, dt, h->b);
    h->launches += 1;
    GB_TRY(check_launch(h, "split source"));
    double bnorm = 0.0;
    GB_TRY(finish_rhs(h, &bnorm));
    GB_CUDA(h, cudaMemcpyAsync(h->p, h->aux[0], h->n0 * sizeof(double),
                               cudaMemcpyDeviceToDevice, s));
    h->stag_mode = nres > 0 ? (restart < nres ? 1 : 2) : 0;
    h->stagnated = false;
    status = solve_internal(h, tol, bnorm, st);
    h->stag_mode = 0;
    cycles += st->cycles;
    if (status != GBMG_OK && status != GBMG_NOT_CONVERGED && status != GBMG_DIVERGED)
      return status;
    if (!h->stagnated) break;
    LAUNCH(h, GBMG_PROF_VECTOR, launch_guess_update(s, h->p, h->aux[0], h->n0, 1.5));
    GB_TRY(check_launch(h, "split restart"));
  }
  h->stagnated = false;
  st->cycles = cycles;
  st->restarts = restart;
  launch_psplit_correct(s, g.nx, g.ny, g.nz, h->rho, h->p, h->aux[0], h->split_rho12, g.dx, g.dy,
                        g.dz, dt, dv[0], dfield[0].sy, dfield[0].sz, dv[1], dfield[1].sy,
                        dfield[1].sz, has_w ? dv[2] : nullptr, has_w ? dfield[2].sy : 0,
                        has_w ? dfield[2].sz : 0);
  h->launches += 1;
  GB_TRY(check_launch(h, "split correction"));
  const int ext[3][3] = {{g.nx + 1, g.ny, g.nz}, {g.nx, g.ny + 1, g.nz}, {g.nx, g.ny, g.nz + 1}};
  if (mem == GBMG_MEM_HOST)
    for (int a = 0; a < 3; ++a) {
      if (a == 2 && !has_w) continue;
      GB_TRY(download(h, dv[a], ext[a][0], ext[a][1], ext[a][2], mem, *fv[a]));
    }
  GB_TRY(download(h, h->p, g.nx, g.ny, g.nz, mem, p));
  GB_CUDA(h, cudaEventRecord(h->ev1, s));
  GB_CUDA(h, cudaEventSynchronize(h->ev1));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, h->ev0, h->ev1);
  st->ms = ms;
  return status;
}

int gbmg_divergence(gbmg_handle* h, gbmg_field u, gbmg_field v, gbmg_field w, double dt,
                    gbmg_field b, int mem) {
  GB_TRY(begin(h));
  GB_TRY(validate_field(h, u, "u"));
  GB_TRY(validate_field(h, v, "v"));
  GB_TRY(validate_field(h, b, "b"));
  const gbmg_grid& g = h->grid;
  const bool has_w = w.data != nullptr && g.nz > 1;
  const int ext[3][3] = {{g.nx + 1, g.ny, g.nz}, {g.nx, g.ny + 1, g.nz}, {g.nx, g.ny, g.nz + 1}};
  const gbmg_field* fv[3] = {&u, &v, &w};
  Strided sd[3] = {{nullptr, 0, 0}, {nullptr, 0, 0}, {nullptr, 0, 0}};
  for (int a = 0; a < 3; ++a) {
    if (a == 2 && !has_w) continue;
    if (mem == GBMG_MEM_DEVICE) {
      sd[a] = Strided{fv[a]->data, fv[a]->sy, fv[a]->sz};
    } else {
      const size_t n = (size_t)ext[a][0] * ext[a][1] * ext[a][2];
      if (h->vel_n[a] < n) {
        dfree(h->vel[a]);
        GB_TRY(dmalloc(h, &h->vel[a], n));
        h->vel_n[a] = n;
      }
      GB_TRY(upload(h, *fv[a], ext[a][0], ext[a][1], ext[a][2], mem, h->vel[a]));
      sd[a] = Strided{h->vel[a], ext[a][0], (int64_t)ext[a][0] * ext[a][1]};
    }
  }
  if (h->prm.zero_wall_faces) {
    const gbmg_field df[3] = {{const_cast<double*>(sd[0].data), sd[0].sy, sd[0].sz},
                              {const_cast<double*>(sd[1].data), sd[1].sy, sd[1].sz},
                              {const_cast<double*>(sd[2].data), sd[2].sy, sd[2].sz}};
    GB_TRY(zero_walls(h, df, has_w));
    if (mem != GBMG_MEM_DEVICE)  // the caller's host arrays get the zeros too
      for (int a = 0; a < 3; ++a) {
        if (a == 2 && !has_w) continue;
        GB_TRY(download(h, sd[a].data, ext[a][0], ext[a][1], ext[a][2], mem, *fv[a]));
      }
  }
  launch_divergence(h->stream, g.nx, g.ny, g.nz, sd[0], sd[1], sd[2], g.dx, g.dy, g.dz, dt, h->b);
  h->launches += 1;
  GB_TRY(check_launch(h, "divergence"));
  GB_TRY(download(h, h->b, g.nx, g.ny, g.nz, mem, b));
  GB_CUDA(h, cudaStreamSynchronize(h->stream));
  return GBMG_OK;
}

int gbmg_residual(gbmg_handle* h, gbmg_field b, gbmg_field p, gbmg_field r, double* norm2,
                  int mem) {
  GB_TRY(begin(h));
  if (!h->coef_ready) { h->err = "no coefficients"; return GBMG_STATE_ERROR; }
  GB_TRY(validate_field(h, b, "b"));
  GB_TRY(validate_field(h, p, "p"));
  const gbmg_grid& g = h->grid;
  GB_TRY(upload(h, b, g.nx, g.ny, g.nz, mem, h->b));
  GB_TRY(upload(h, p, g.nx, g.ny, g.nz, mem, h->p));
  Level& f = h->lv[0];
  f.sol = h->p; f.src = h->b;
  // the residual overwrites the staging copy of b (not the caller's array)
  launch_residual_norm<double>(h->stream, v64(f), r.data ? h->b : nullptr, h->red, kSlotNorm);
  h->launches += 1;
  GB_TRY(check_launch(h, "residual"));
  double s2 = 0.0;
  GB_TRY(read_result(h, kSlotNorm, &s2));
  if (norm2) *norm2 = s2;
  if (r.data) {
    GB_TRY(download(h, h->b, g.nx, g.ny, g.nz, mem, r));
    GB_CUDA(h, cudaStreamSynchronize(h->stream));
  }
  return GBMG_OK;
}

int gbmg_div_stats(gbmg_handle* h, gbmg_field u, gbmg_field v, gbmg_field w, double* max_div,
                   double* mean_div, int mem) {
  GB_TRY(begin(h));
  GB_TRY(validate_field(h, u, "u"));
  GB_TRY(validate_field(h, v, "v"));
  const gbmg_grid& g = h->grid;
  const bool has_w = w.data != nullptr && g.nz > 1;
  const int ext[3][3] = {{g.nx + 1, g.ny, g.nz}, {g.nx, g.ny + 1, g.nz}, {g.nx, g.ny, g.nz + 1}};
  const gbmg_field* fv[3] = {&u, &v, &w};
  Strided sd[3] = {{nullptr, 0, 0}, {nullptr, 0, 0}, {nullptr, 0, 0}};
  for (int a = 0; a < 3; ++a) {
    if (a == 2 && !has_w) continue;
    if (mem == GBMG_MEM_DEVICE) {
      sd[a] = Strided{fv[a]->data, fv[a]->sy, fv[a]->sz};
    } else {
      const size_t n = (size_t)ext[a][0] * ext[a][1] * ext[a][2];
      if (h->vel_n[a] < n) {
        dfree(h->vel[a]);
        GB_TRY(dmalloc(h, &h->vel[a], n));
        h->vel_n[a] = n;
      }
      GB_TRY(upload(h, *fv[a], ext[a][0], ext[a][1], ext[a][2], mem, h->vel[a]));
      sd[a] = Strided{h->vel[a], ext[a][0], (int64_t)ext[a][0] * ext[a][1]};
    }
  }
  launch_div_stats(h->stream, g.nx, g.ny, g.nz, sd[0], sd[1], sd[2], g.dx, g.dy, g.dz, h->red);
  h->launches += 1;
  GB_TRY(check_launch(h, "div_stats"));
  double sum = 0.0;
  GB_TRY(read_result(h, kSlotSum, &sum));
  if (max_div) *max_div = h->host_res[kSlotMax];
  if (mean_div) *mean_div = sum / (double)h->n0;
  return GBMG_OK;
}

int gbmg_adjoint(gbmg_handle* h, gbmg_field p, gbmg_field lam, gbmg_field phi, double eps,
                 double rho_pos, double rho_neg, gbmg_field grad_rho, gbmg_field grad_phi,
                 int mem) {
  GB_TRY(begin(h));
  if (!h->rho_ready) { h->err = "the adjoint needs the density: call gbmg_set_rho/phi first"; return GBMG_STATE_ERROR; }
  GB_TRY(validate_field(h, p, "p"));
  GB_TRY(validate_field(h, lam, "lam"));
  GB_TRY(validate_field(h, grad_rho, "grad_rho"));
  const bool want_phi = phi.data != nullptr;
  if (want_phi) {
    GB_TRY(validate_field(h, grad_phi, "grad_phi"));
    if (!(eps > 0)) { h->err = "eps must be > 0"; return GBMG_INVALID_ARG; }
  }
  const gbmg_grid& g = h->grid;
  for (int a = 0; a < 2; ++a)
    if (!h->aux[a]) GB_TRY(dmalloc(h, &h->aux[a], h->n0));
  // p -> h->p, lam -> h->b (both staging copies), phi -> aux[1] if in host memory
  GB_TRY(upload(h, p, g.nx, g.ny, g.nz, mem, h->p));
  GB_TRY(upload(h, lam, g.nx, g.ny, g.nz, mem, h->b));
  Strided sp{nullptr, 0, 0};
  if (want_phi) {
    if (mem == GBMG_MEM_HOST) {
      GB_TRY(upload(h, phi, g.nx, g.ny, g.nz, mem, h->aux[1]));
      sp = Strided{h->aux[1], g.nx, (int64_t)g.nx * g.ny};
    } else {
      sp = Strided{phi.data, phi.sy, phi.sz};
    }
  }
  double* gphi = want_phi ? h->aux[1] : nullptr;
  // when phi lives in aux[1] (host input), the kernel reads and writes the same
  // cell only, so grad_phi may overwrite it in place
  LAUNCH(h, GBMG_PROF_VECTOR,
         launch_adjoint(h->stream, g.nx, g.ny, g.nz, g.dx * g.dx, g.dy * g.dy, g.dz * g.dz, h->rho,
                        h->p, h->b, sp, eps, rho_pos, rho_neg, h->aux[0], gphi));
  GB_TRY(check_launch(h, "adjoint"));
  GB_TRY(download(h, h->aux[0], g.nx, g.ny, g.nz, mem, grad_rho));
  if (want_phi) GB_TRY(download(h, h->aux[1], g.nx, g.ny, g.nz, mem, grad_phi));
  GB_CUDA(h, cudaStreamSynchronize(h->stream));
  return GBMG_OK;
}

int gbmg_level_coef(gbmg_handle* h, int level, gbmg_field cx, gbmg_field cy, gbmg_field cz,
                    int mem) {
  GB_TRY(begin(h));
  if (!h->coef_ready) { h->err = "no coefficients"; return GBMG_STATE_ERROR; }
  if (level < 0 || level >= h->L) return GBMG_INVALID_ARG;
  const Level& v = h->lv[level];
  GB_TRY(download(h, v.cx, v.nx, v.ny, v.nz, mem, cx));
  GB_TRY(download(h, v.cy, v.nx, v.ny, v.nz, mem, cy));
  GB_TRY(download(h, v.cz, v.nx, v.ny, v.nz, mem, cz));
  GB_CUDA(h, cudaStreamSynchronize(h->stream));
  return GBMG_OK;
}

int gbmg_level_dims(gbmg_handle* h, int32_t* levels, int32_t* dims, int32_t max_levels) {
  if (!h) return GBMG_INVALID_ARG;
  if (levels) *levels = h->L;
  if (dims)
    for (int l = 0; l < h->L && l < max_levels; ++l) {
      dims[3 * l] = h->lv[l].nx;
      dims[3 * l + 1] = h->lv[l].ny;
      dims[3 * l + 2] = h->lv[l].nz;
    }
  return GBMG_OK;
}

int64_t gbmg_kernel_launches(gbmg_handle* h) { return h ? h->launches : 0; }

int gbmg_set_profiling(gbmg_handle* h, int on) {
  GB_TRY(begin(h));
  prof_flush(h);
  h->prof = on != 0;
  for (int c = 0; c < GBMG_PROF_CLASSES; ++c) {
    h->prof_ms[c] = 0.0;
    h->prof_n[c] = 0;
  }
  return GBMG_OK;
}


int gbmg_profile(gbmg_handle* h, double* ms, int64_t* launches, int32_t n) {
  GB_TRY(begin(h));
  prof_flush(h);
  for (int c = 0; c < GBMG_PROF_CLASSES && c < n; ++c) {
    if (ms) ms[c] = h->prof_ms[c];
    if (launches) launches[c] = h->prof_n[c];
  }
  return GBMG_OK;
}

const char* gbmg_strerror(int status) {
  switch (status) {
    case GBMG_OK: return "ok";
    case GBMG_NOT_CONVERGED: return "not converged within max_cycles";
    case GBMG_DIVERGED: return "diverged (residual not finite or grew 1e3-fold)";
    case GBMG_INVALID_ARG: return "invalid argument";
    case GBMG_CUDA_ERROR: return "CUDA error";
    case GBMG_NO_DEVICE: return "no CUDA device";
    case GBMG_OUT_OF_MEMORY: return "out of device memory";
    case GBMG_STATE_ERROR: return "call out of order";
    default: return "unknown status";
  }
}

const char* gbmg_last_error(gbmg_handle* h) { return h ? h->err.c_str() : ""; }

}  // extern "C"
